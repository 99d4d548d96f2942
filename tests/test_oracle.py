"""The CPU oracle pinned against the reference's own known-answer vectors and
against values computed by the unmodified reference library (fixtures)."""
import math

import numpy as np
import pytest

from conftest import rel, relx
from oracle import binding as ob

CLIGHT = 299792458.0


def test_mie_perf_golden(unit_vectors):
    t = unit_vectors["test_mie_perf"]
    for c in t["cases"]:
        a, b = ob.mie(c["LbyR"], c["xi"], c["l"], math.inf)
        assert relx(a, c["lna"]) < t["tolerance"], c
        assert relx(b, c["lnb"]) < t["tolerance"], c


def test_mie_drude_golden(unit_vectors):
    t = unit_vectors["test_mie_drude"]
    for c in t["cases"]:
        R, L = c["R"], c["L"]
        wp, gam = c["omegap_scaled"] * CLIGHT / (L + R), c["gamma_scaled"] * CLIGHT / (L + R)
        xi = c["xi"] * CLIGHT / (L + R)
        eps = wp * wp / (xi * (xi + gam))
        a, b = ob.mie(L / R, c["xi"], c["l"], eps)
        assert relx(a, c["lna"]) < t["tolerance"], c
        assert relx(b, c["lnb"]) < t["tolerance"], c


def test_mie_grid_reference(ref_values):
    for c in ref_values["mie_grid"]:
        R, L = c["R"], c["L"]
        if c["drude"]:
            xi = c["xi"] * CLIGHT / (L + R)
            wp, gam = c["drude"][0] / ob.HBAR_EV, c["drude"][1] / ob.HBAR_EV
            eps = wp * wp / (xi * (xi + gam))
        else:
            eps = math.inf
        a, b = ob.mie(L / R, c["xi"], c["l"], eps)
        assert relx(a, c["lna"]) < 1e-12 and relx(b, c["lnb"]) < 1e-12, c


@pytest.mark.parametrize("name", ["pr_RbyL20_ldim140", "drude_RbyL20_ldim140", "drude_RbyL150_ldim80"])
def test_logdetD_reference(ref_values, name):
    for c in ref_values[name]:
        v = ob.logdetD(c["R"], c["L"], c["ldim"], c["xi"], c["m"], c["drude"])
        assert rel(v, c["LU"]) < 1e-11, (c, v)
        assert rel(v, c["HODLR"]) < 1e-10, (c, v)


def test_dense_M_reference(ref_values):
    for c in ref_values["dense_M"]:
        M = ob.M_dense(c["R"], c["L"], c["ldim"], c["xi"], c["m"], c["drude"])
        Mr = np.array(c["M"])
        scale = np.abs(Mr).max()
        # elements agree to ~1e-12 of the largest element (reference K integrals carry epsrel=1e-8 QUADPACK error)
        assert np.abs(M - Mr).max() < 5e-12 * scale, c["m"]


def test_I_reference(ref_values):
    import ctypes as C
    for c in ref_values["K_I"][:2]:
        g = ob.geom(c["R"], c["L"], c["ldim"], c["drude"])
        for l1, l2, p, v, s in c["I"]:
            sg = C.c_int()
            w = ob.lib.oracle_I(C.byref(g), c["xi"], c["m"], l1, l2, p, C.byref(sg))
            if s == 0:
                assert sg.value == 0
                continue
            assert sg.value == s and abs(w - v) < 1e-11 * max(1, abs(v)), (l1, l2, p, v, w)


def test_lnLambda_symmetry():
    for l1, l2, m in [(1, 1, 0), (5, 9, 3), (300, 1200, 200), (2000, 2100, 1000)]:
        assert ob.lib.oracle_lnLambda(l1, l2, m) == ob.lib.oracle_lnLambda(l2, l1, m)


def test_ht_drude_limit():
    # Drude high-temperature term is negative and grows with R/L
    a, b = ob.lib.oracle_ht_drude(1 / 20), ob.lib.oracle_ht_drude(1 / 150)
    assert b < a < 0


def test_ht_plasma_golden(unit_vectors):
    """the plasma-model xi=0 free energy against the reference's own vectors
    (src/tests/test_logdetD.c:121-126, 1e-10)"""
    t = unit_vectors["test_logdetD0"]
    for c in t["ht_plasma"]:
        got = ob.ht_plasma(c["R"], c["L"], c["ldim"], c["omegap_scaled"], c["eps"])
        assert abs(got - c["ht_plasma"]) <= t["tolerance"] * abs(c["ht_plasma"]), (c, got)


def test_plasma_I_limits():
    """I_nu is an average of -r_TE over a Gamma(nu+1) density: in (0,1), increasing
    with omegap, and 1 - I_nu ~ nu/omegap for omegap >> nu (-r_TE ~ 1 - t/omegap)"""
    for nu in (2, 17, 300):
        vals = [ob.plasma_I(nu, w) for w in (0.01, 1.0, 100.0, 1e5)]
        assert all(0 < v < 1 for v in vals)
        assert vals == sorted(vals)
        assert 1 - vals[-1] < 4 * (nu + 1) / 1e5


@pytest.mark.parametrize("name", ["pr_RbyL10_ldim70_T300", "drude_RbyL10_ldim70_T300", "plasma_RbyL10_ldim70_T300"])
def test_free_energy_golden(energy_golden, name):
    """the oracle's Matsubara sum (incl. the xi=0 rule of each material model) against the
    reference library run through the serial restatement of its driver"""
    d = energy_golden[name]
    drude = tuple(d["drude"]) if d["drude"] else None
    E, info = ob.free_energy(d["R"], d["L"], d["ldim"], d["T"], drude, threads=8)
    assert info["nxi"] == len(d["xi"])
    assert abs(E - d["E"]) <= 1e-10 * abs(d["E"]), (E, d["E"])
    assert abs(info["logdetD"][0] - d["logdetD"][0]) <= 1e-10 * abs(d["logdetD"][0])
