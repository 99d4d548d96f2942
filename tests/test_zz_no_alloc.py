"""The allocation-free entry point caps_logdetD_noalloc.

caps_logdetD_noalloc serves callers that may not allocate device memory while
they run -- a framework that owns the whole device through its own pool
allocator, where an outside cudaMalloc can fail or fragment the pool.  Its
scratch is a fixed file-scope device array shared by every call.  Its results
are checked against caps_logdetD (the allocating entry point), against the
reference library's values (tests/golden/reference_values.json, computed by
the unmodified CaPS library) and against the CPU oracle, on calls in a row, so
that a fault shared with the allocating path is also caught.  This file is
collected last so that a run stopping at the first failure has run every other
test first; it also passes alone in a fresh process.
"""
import ctypes as C

import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _noalloc(cg, caps, xi_, m):
    out = C.c_double(float("nan"))
    rc = cg.lib.caps_logdetD_noalloc(caps._h, float(xi_), int(m), C.byref(out))
    return rc, out.value


def test_noalloc_matches_logdetD_two_calls():
    import caps_gb300 as cg
    a = cg.Caps(20e-6, 1e-6, ldim=140, detalg=cg.DETALG_LU)
    b = cg.Caps(50e-6, 1e-6, ldim=120)          # default (HODLR) semantics
    b.set_drude(9.0, 0.035)
    cases = [(a, 1.0, 3), (b, 7.5, 12)]
    # the two calls in a row share (and reuse) the scratch array
    got = [_noalloc(cg, c, xi, m) for c, xi, m in cases]
    for (c, xi, m), (rc, v) in zip(cases, got):
        assert rc == 0, cg.lib.caps_noalloc_last_error()
        want = c.logdetD(xi, m)
        assert rel(v, want) < TOL, (xi, m, v, want)
    # repeat the first call after the second: stale contents must not matter
    rc, v = _noalloc(cg, a, 1.0, 3)
    assert rc == 0 and v == got[0][1]


@pytest.mark.parametrize("name", ["pr_RbyL20_ldim140", "drude_RbyL20_ldim140"])
def test_noalloc_matches_reference_library(ref_values, name):
    """every case of the fixture set, in a row, against the reference library's LU and
    HODLR values at the plain form's bar"""
    import caps_gb300 as cg
    for v in ref_values[name]:
        for detalg, key in ((cg.DETALG_LU, "LU"), (cg.DETALG_HODLR, "HODLR")):
            c = cg.Caps(v["R"], v["L"], ldim=v["ldim"], detalg=detalg)
            if v["drude"]:
                c.set_drude(*v["drude"])
            rc, got = _noalloc(cg, c, v["xi"], v["m"])
            assert rc == 0, cg.lib.caps_noalloc_last_error()
            assert rel(got, v[key]) < TOL, (name, v["xi"], v["m"], key, got, v[key])


def test_noalloc_matches_oracle():
    """a geometry with no fixture (R/L=35, Drude) against the CPU oracle"""
    import caps_gb300 as cg
    from oracle import binding as ob
    R, L, ldim = 35e-6, 1e-6, 90
    c = cg.Caps(R, L, ldim=ldim, detalg=cg.DETALG_LU)
    c.set_drude(8.0, 0.04)
    for xi_, m in ((2.0, 0), (2.0, 9), (15.0, 4)):
        rc, got = _noalloc(cg, c, xi_, m)
        assert rc == 0, cg.lib.caps_noalloc_last_error()
        want = ob.logdetD(R, L, ldim, xi_, m, drude=(8.0, 0.04))
        assert rel(got, want) < TOL, (xi_, m, got, want)


def test_noalloc_rejects_oversize():
    import caps_gb300 as cg
    c = cg.Caps(150e-6, 1e-6, ldim=1050)
    rc, v = _noalloc(cg, c, 1.0, 0)
    assert rc < 0
    assert "ldim" in cg.lib.caps_noalloc_last_error().decode()
