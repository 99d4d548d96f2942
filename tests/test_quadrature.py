"""The frequency-integration rules of the T=0 and PSD drivers, on host callbacks and
without a GPU, against the reference's own dqagi (cquadpack), fcqs_semiinf (src/fcqs.c)
and psd (src/psd.c) results recorded in tests/golden/quad_golden.json: the same
algorithm must give the same abscissae, decisions and results."""
import ctypes as C
import json
import math
import os

import pytest

import quad_cases as Q

HERE = os.path.dirname(os.path.abspath(__file__))
FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)


@pytest.fixture(scope="module")
def golden():
    return json.load(open(os.path.join(HERE, "golden", "quad_golden.json")))


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("b", os.path.join(os.path.dirname(HERE), "caps_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    if not os.path.exists(b.LIB):
        pytest.skip("library not built")
    L = C.CDLL(b.LIB)
    d, i = C.c_double, C.c_int
    L.caps_dqagi.restype = d
    L.caps_dqagi.argtypes = [FN, C.c_void_p, d, i, d, d, C.POINTER(d), C.POINTER(i), C.POINTER(i)]
    L.caps_fcqs_semiinf.restype = d
    L.caps_fcqs_semiinf.argtypes = [FN, C.c_void_p, C.POINTER(d), C.POINTER(i), d, C.POINTER(i)]
    L.caps_psd.restype = i
    L.caps_psd.argtypes = [i, C.POINTER(d), C.POINTER(d)]
    return L


@pytest.mark.parametrize("name", sorted(Q.QAGI))
@pytest.mark.parametrize("eps", Q.EPSRELS)
def test_qagi_matches_reference(lib, golden, name, eps):
    f, bound, inf = Q.QAGI[name]
    cb = FN(lambda x, _u: f(x))
    ab, ne, ier = C.c_double(), C.c_int(), C.c_int()
    r = lib.caps_dqagi(cb, None, bound, inf, 0.0, eps, C.byref(ab), C.byref(ne), C.byref(ier))
    g = golden["qagi"]["%s_%g" % (name, eps)]
    assert (ne.value, ier.value) == (g["neval"], g["ier"])
    assert r == g["result"] and ab.value == g["abserr"], (r, g)


@pytest.mark.parametrize("name", sorted(Q.FCQS))
def test_fcqs_matches_reference(lib, golden, name):
    f, L = Q.FCQS[name]
    cb = FN(lambda x, _u: f(x))
    eps, ne, ier = C.c_double(1e-10), C.c_int(), C.c_int()
    r = lib.caps_fcqs_semiinf(cb, None, C.byref(eps), C.byref(ne), L, C.byref(ier))
    g = golden["fcqs"][name]
    assert (ne.value, ier.value) == (g["neval"], g["ier"])
    assert r == g["result"] and eps.value == g["epsrel"], (r, g)


def test_psd_matches_reference(lib, golden):
    """poles and weights of the Pade spectrum decomposition: LAPACK dstemr in the
    reference, Sturm bisection here.  The bar is dstemr's own accuracy: its poles carry
    up to ~2e-13 relative error (see the next test), which the weights amplify to ~1e-11
    at order 64."""
    for N, g in golden["psd"].items():
        N = int(N)
        xi, eta = (C.c_double * N)(), (C.c_double * N)()
        assert lib.caps_psd(N, xi, eta) == 0
        for k in range(N):
            assert abs(xi[k] - g["xi"][k]) <= 5e-13 * abs(g["xi"][k]), (N, k, xi[k], g["xi"][k])
            assert abs(eta[k] - g["eta"][k]) <= 5e-11 * abs(g["eta"][k]), (N, k, eta[k], g["eta"][k])


def test_psd_low_poles_are_matsubara(lib):
    """for large order the lowest PSD poles converge to the Matsubara frequencies 2 pi k
    (Hu, Xu, Yan 2010) with weights -> 1: the bisection reaches them to rounding"""
    N = 40
    xi, eta = (C.c_double * N)(), (C.c_double * N)()
    lib.caps_psd(N, xi, eta)
    for k in range(5):
        assert abs(xi[k] / (2 * math.pi * (k + 1)) - 1) < 4e-16, (k, xi[k])
        assert abs(eta[k] - 1) < 1e-14, (k, eta[k])


def test_gauss_laguerre_rule():
    """caps_gauss_laguerre (the T = 0 Gauss-Laguerre driver's rule): numpy's nodes and weights,
    and the moments int_0^inf e^-x x^k dx = k! exact for k <= 2n - 1"""
    import math

    import numpy as np

    import caps_gb300 as cg
    for n in (5, 20, 60):
        x, wex = cg.gauss_laguerre(n)
        xr, wr = np.polynomial.laguerre.laggauss(n)
        assert np.max(np.abs(x - xr) / xr) < 1e-12
        assert np.max(np.abs(wex * np.exp(-x) - wr) / wr) < 1e-10
        for k in (0, 1, n, 2 * n - 1):
            s = sum(math.exp(math.log(wi) - xi + k * math.log(xi)) for xi, wi in zip(x, wex))
            assert abs(s / math.factorial(k) - 1) < 1e-11, (n, k, s)
