"""The benchmark workloads' free energies against the reference library's own runs of
them (tests/golden/make_golden_energy.py: the serial restatement of the caps driver's
Matsubara loop, src/caps.c:307-396 and :836-849, around the unmodified libcaps):

  * perfect reflectors, R/L = 50, ldim 350, T = 300 K (577 matrices of dimension 700
    and the xi = 0 term from 54 matrices of dimension 350);
  * Drude gold (omega_p = 9 eV, gamma = 0.035 eV), R/L = 150, ldim 1050, T = 300 K
    (978 matrices of dimension 2100), with every per-matrix value of the reference.

Bars: the plain FP64 form at |dE/E| <= 1e-10 and per matrix |d logdetD| <= 1e-10
max(1, |logdetD|); the mixed form with learned truncation at |dE/E| <= 1e-6 (the
required bar) and per matrix 5e-8 max(1, |logdetD|)."""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
HBAR, KB, CL = 1.0545718e-34, 1.38064852e-23, 299792458.0


def golden(name):
    return json.load(open(os.path.join(GOLDEN, "energy_%s.json" % name)))


def caps_for(cg, d, prec):
    c = cg.Caps(d["R"], d["L"], ldim=d["ldim"], detalg=cg.DETALG_LU)
    if d["drude"]:
        c.set_drude(*d["drude"])
    c.set_precision(prec)
    return c


@pytest.fixture(scope="module")
def cg():
    import caps_gb300
    return caps_gb300


@pytest.fixture(scope="module")
def held_out_net():
    """the network of the benchmark: trained on R/L <= 50 and Drude metals other than gold"""
    from caps_gb300 import learned
    net, info = learned.train(seed=0)
    assert 150.0 not in info["geometries_RbyL"] and (9.0, 0.035) not in info["materials"]
    return net


@pytest.mark.parametrize("name", ["pr_RbyL50_ldim350_T300", "drude_RbyL150_ldim1050_T300"])
def test_free_energy_fp64(cg, name):
    d = golden(name)
    c = caps_for(cg, d, cg.PREC_FP64)
    E, info = c.free_energy(d["T"], d["cutoff"], d["epsrel"])
    assert info["nxi"] == len(d["xi"]), (info, len(d["xi"]))
    if d["drude"]:   # (perfect reflectors also count the matrices of the xi = 0 term)
        assert info["ndet"] - info["nwasted"] == d["ndet"], (info, d["ndet"])
    assert abs(E - d["E"]) <= 1e-10 * abs(d["E"]), (E, d["E"])
    for k, (got, want) in enumerate(zip(info["logdetD"], d["logdetD"])):
        assert abs(got - want) <= 1e-10 * max(1.0, abs(want)), (k, got, want)


@pytest.mark.parametrize("name", ["pr_RbyL50_ldim350_T300", "drude_RbyL150_ldim1050_T300"])
def test_free_energy_mixed_learned(cg, held_out_net, name):
    """the chosen form: mixed precision with the learned proposal (network held out from the
    workload) equals the plain mixed form exactly and the reference within 1e-6"""
    d = golden(name)
    c = caps_for(cg, d, cg.PREC_MIXED)
    E1, i1 = c.free_energy(d["T"], d["cutoff"], d["epsrel"], mlp=held_out_net)
    E0, i0 = c.free_energy(d["T"], d["cutoff"], d["epsrel"])
    assert E1 == E0, (E1, E0)
    assert i1["ndet"] - i1["nwasted"] == i0["ndet"] - i0["nwasted"]
    if d["drude"]:
        assert i1["ndet"] - i1["nwasted"] == d["ndet"]
    err = abs(E1 - d["E"]) / abs(d["E"])
    assert err <= 1e-6, (E1, d["E"], err)
    print("%s: |dE/E| = %.2e, matrices %d (learned) vs %d (plain), reference %d" %
          (name, err, i1["ndet"], i0["ndet"], d["ndet"]))


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 5e-8)])
def test_every_matrix_of_the_r150_workload(cg, prec, tol):
    """each of the 978 logdetD of the R/L = 150 free energy against the reference's value"""
    d = golden("drude_RbyL150_ldim1050_T300")
    Ts = 2 * math.pi * KB * (d["R"] + d["L"]) * d["T"] / (HBAR * CL)
    xi = [(k + 1) * Ts for k, t in enumerate(d["terms"]) for _ in t]
    ms = [m for t in d["terms"] for m in range(len(t))]
    want = np.array([v for t in d["terms"] for v in t])
    c = caps_for(cg, d, cg.PREC_MIXED if prec == "mixed" else cg.PREC_FP64)
    got, st = c.logdetD_batch(xi, ms)
    assert max(st) < 16
    e = np.abs(np.array(got) - want) / np.maximum(1.0, np.abs(want))
    print("%s: per-matrix error max %.2e, p99 %.2e over %d matrices" % (prec, e.max(), np.percentile(e, 99), len(e)))
    assert e.max() <= tol, (int(e.argmax()), e.max())
