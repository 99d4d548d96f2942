"""The batched HODLR path (hodlr.cu: adaptive cross approximation with rook pivoting, the
elements evaluated on demand, the symmetric HODLR factorisation) against the reference's
HODLR and LU values and against the dense GPU path.

Bars: |d logdetD| <= 1e-10 max(1, |logdetD|), the reference's own test tolerance
(src/tests/test_logdetD.c:57), against the values the reference library computes with its
HODLR (libhodlr) and LU determinants."""
import time

import pytest

from conftest import rel, relx

pytestmark = pytest.mark.gpu
TOL = 1e-10


@pytest.fixture(scope="module")
def cg():
    import caps_gb300
    return caps_gb300


def caps(cg, R, L, ldim, drude=None, path=None):
    c = cg.Caps(R, L, ldim=ldim)          # DETALG_HODLR, FP64
    if drude:
        c.set_drude(*drude)
    if path is not None:
        assert cg.lib.caps_gpu_set_path(c._h, path) == 1
    return c


@pytest.mark.parametrize("name", ["pr_RbyL20_ldim140", "drude_RbyL20_ldim140", "pr_RbyL50_ldim350", "drude_RbyL150_ldim1050"])
def test_hodlr_vs_reference_fixtures(cg, ref_values, name):
    """the HODLR path forced on every fixture of the reference library (its HODLR and LU
    values) in one batch per geometry"""
    cases = ref_values[name]
    c0 = cases[0]
    c = caps(cg, c0["R"], c0["L"], c0["ldim"], c0["drude"], cg.PATH_HODLR)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    for v, got, s in zip(cases, out, st):
        assert s < 16, (v, s)
        assert rel(got, v["HODLR"]) < TOL, (name, v["xi"], v["m"], got, v["HODLR"])
        assert rel(got, v["LU"]) < TOL, (name, v["xi"], v["m"], got, v["LU"])


def test_hodlr_equals_dense_path(cg):
    """one batch, HODLR against the dense Cholesky with the same result rules, Drude R/L=50"""
    xi = [41.98, 41.98, 41.98, 125.9, 125.9, 300.0]
    ms = [0, 7, 30, 2, 45, 11]
    h = caps(cg, 50e-6, 1e-6, 350, (9.0, 0.035), cg.PATH_HODLR).logdetD_batch(xi, ms)[0]
    d = caps(cg, 50e-6, 1e-6, 350, (9.0, 0.035), cg.PATH_DENSE).logdetD_batch(xi, ms)[0]
    for x, m, a, b in zip(xi, ms, h, d):
        assert rel(a, b) < TOL, (x, m, a, b)


def test_hodlr_unit_vectors_RbyL100(cg, unit_vectors):
    """src/tests/test_logdetD.c:13-76 (R/L=100, ldim 500, the reference's default HODLR) by
    the HODLR path"""
    t = unit_vectors["test_logdetD"]
    cases = [v for v in t["cases"] if v["ldim"] == 500]
    c = caps(cg, 1.0, 0.01, 500, None, cg.PATH_HODLR)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    for v, got, s in zip(cases, out, st):
        assert s < 16
        assert relx(got, v["logdetD"]) < t["tolerance"], (v, got)


def test_hodlr_unit_vectors_RbyL1000(cg, unit_vectors):
    """src/tests/test_logdetD.c:77-102 (R/L=1000, ldim 10000, matrices of dimension 20000):
    the automatic path takes HODLR at this size; against the dense FP64 time"""
    t = unit_vectors["test_logdetD"]
    cases = [v for v in t["cases"] if v["ldim"] == 10000]
    c = caps(cg, 1.0, 0.001, 10000)
    t0 = time.time()
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    th = time.time() - t0
    for v, got, s in zip(cases, out, st):
        assert s < 16, (v, s)
        assert relx(got, v["logdetD"]) < t["tolerance"], (v, got)
    print("R/L=1000, dimension 20000: %d matrices by HODLR in %.2f s" % (len(cases), th))


def test_large_aspect_workload_vs_reference(cg):
    """plasma, R/L = 1000, L = 100 nm, ldim 6000 (dimension 12000) at three nodes of the
    60-point Gauss-Laguerre rule (tests/golden/reference_c4.json, the reference library's LU
    and HODLR values): the FP64 form (automatic path: HODLR) at 1e-10, the mixed form at 5e-8"""
    import json
    import os

    from conftest import GOLDEN
    d = json.load(open(os.path.join(GOLDEN, "reference_c4.json")))
    cases = d["cases"]
    v0 = cases[0]
    for prec, tol in ((cg.PREC_FP64, TOL), (cg.PREC_MIXED, 5e-8)):
        c = caps(cg, v0["R"], v0["L"], v0["ldim"], (v0["omegap_eV"], v0["gamma_eV"]))
        c.set_precision(prec)
        out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
        for v, got, s in zip(cases, out, st):
            assert s < 16, (v, s)
            assert rel(got, v["LU"]) < tol, (prec, v["xi"], v["m"], got, v["LU"])
            assert rel(got, v["HODLR"]) < tol, (prec, v["xi"], v["m"], got, v["HODLR"])


def test_hodlr_free_energy_T0_gauss_laguerre(cg):
    """a T = 0 free energy (20-point Gauss-Laguerre rule, plasma, R/L = 100, L = 100 nm,
    dimension 1400) through the HODLR path equals the dense FP64 path's to 1e-10"""
    E = {}
    for path in (cg.PATH_HODLR, cg.PATH_DENSE):
        c = caps(cg, 1e-5, 1e-7, 700, (9.0, 0.0), path)
        E[path], info = c.free_energy_T0_gl(20)
        assert info["ndet"] > 0
    assert abs(E[cg.PATH_HODLR] - E[cg.PATH_DENSE]) <= 1e-10 * abs(E[cg.PATH_DENSE]), E


@pytest.mark.parametrize("name", ["pr_RbyL50_ldim350", "drude_RbyL150_ldim1050"])
def test_mixed_hodlr_vs_reference_fixtures(cg, ref_values, name):
    """the mixed form's HODLR path (float-float sampled elements, FP64 compression and
    factorisation) against the reference library's HODLR and LU values at the mixed bar"""
    cases = ref_values[name]
    c0 = cases[0]
    c = caps(cg, c0["R"], c0["L"], c0["ldim"], c0["drude"], cg.PATH_HODLR)
    c.set_precision(cg.PREC_MIXED)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    for v, got, s in zip(cases, out, st):
        assert s < 16, (v, s)
        assert rel(got, v["HODLR"]) < 5e-8, (name, v["xi"], v["m"], got, v["HODLR"])
        assert rel(got, v["LU"]) < 5e-8, (name, v["xi"], v["m"], got, v["LU"])


def test_mixed_hodlr_large_aspect_vs_reference(cg):
    """dimension 12000 (plasma, R/L = 1000, L = 100 nm): the mixed HODLR path against the
    reference library's values at the mixed bar"""
    import json
    import os

    from conftest import GOLDEN
    cases = json.load(open(os.path.join(GOLDEN, "reference_c4.json")))["cases"]
    v0 = cases[0]
    c = caps(cg, v0["R"], v0["L"], v0["ldim"], (v0["omegap_eV"], v0["gamma_eV"]), cg.PATH_HODLR)
    c.set_precision(cg.PREC_MIXED)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    worst = 0.0
    for v, got, s in zip(cases, out, st):
        assert s < 16, (v, s)
        worst = max(worst, rel(got, v["LU"]))
        assert rel(got, v["LU"]) < 5e-8, (v["xi"], v["m"], got, v["LU"])
    print("mixed HODLR, dimension 12000: largest error against the reference's LU %.1e" % worst)
