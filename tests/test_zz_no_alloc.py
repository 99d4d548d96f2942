"""The allocation-free entry point caps_logdetD_noalloc against caps_logdetD.

caps_logdetD_noalloc serves callers that may not allocate device memory while
they run (a framework owning the device through its own pool, or code inside a
stream capture): its scratch is a fixed file-scope device array.  This file is
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


def test_noalloc_rejects_oversize():
    import caps_gb300 as cg
    c = cg.Caps(150e-6, 1e-6, ldim=1050)
    rc, v = _noalloc(cg, c, 1.0, 0)
    assert rc < 0
    assert "ldim" in cg.lib.caps_noalloc_last_error().decode()
