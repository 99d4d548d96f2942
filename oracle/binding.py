"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

Test infrastructure only: imported by tests/, by __graft_entry__.smoke() and by
bench.py's CPU-baseline leg, always as the parity reference or the timed baseline.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
HBAR_EV = 6.582119514e-16
PERFECT, DRUDE = 0, 1


class Material(C.Structure):
    _fields_ = [("kind", C.c_int), ("omegap", C.c_double), ("gamma", C.c_double)]


class Geom(C.Structure):
    _fields_ = [("R", C.c_double), ("L", C.c_double), ("ldim", C.c_int), ("plate", Material), ("sphere", Material)]


def _load():
    if not os.path.exists(LIB_PATH):
        import importlib.util
        spec = importlib.util.spec_from_file_location("caps_gb300_build", os.path.join(os.path.dirname(HERE), "caps_gb300", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build_oracle()
    lib = C.CDLL(LIB_PATH)
    d, i, dp, gp = C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(Geom)
    sig = {
        "oracle_mie": (None, [d, d, i, d, dp, dp]),
        "oracle_lnLambda": (d, [i, i, i]),
        "oracle_lmin": (i, [d, i, i]),
        "oracle_lnPlm": (d, [i, i, d]),
        "oracle_logIK_half": (None, [i, d, dp, dp]),
        "oracle_ratioI": (d, [d, d]),
        "oracle_logdetD": (d, [gp, d, i]),
        "oracle_M_dense": (None, [gp, d, i, dp]),
        "oracle_K_table": (None, [gp, d, i, i, i, dp, dp]),
        "oracle_I": (d, [gp, d, i, i, i, i, C.POINTER(C.c_int)]),
        "oracle_ht_drude": (d, [d]),
        "oracle_logdetD0_MM": (d, [gp, i]),
        "oracle_ht_perf": (d, [gp, d]),
        "oracle_plasma_I": (d, [i, d]),
        "oracle_logdetD0_MM_plasma": (d, [gp, i, d]),
        "oracle_ht_plasma": (d, [gp, d, d]),
        "oracle_logdetD_batch": (None, [gp, i, dp, C.POINTER(C.c_int), dp, i]),
        "oracle_free_energy": (d, [gp, d, d, d, i, dp, dp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
        "oracle_logdet_1mM": (d, [dp, i, C.POINTER(C.c_int)]),
        "oracle_bessel_logI0": (d, [d]),
        "oracle_bessel_logI1": (d, [d]),
        "oracle_bessel_logK0": (d, [d]),
        "oracle_bessel_logK1": (d, [d]),
        "oracle_bessel_logIn": (d, [i, d]),
        "oracle_bessel_logKn": (d, [i, d]),
        "oracle_capc_logdet": (d, [d, d, i, d, C.c_char, i]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype, f.argtypes = r, a
    return lib


lib = _load()


def geom(R, L, ldim, drude=None):
    """drude = (omegap_eV, gamma_eV) for plate and sphere, None for perfect reflectors."""
    if drude:
        mat = Material(DRUDE, drude[0] / HBAR_EV, drude[1] / HBAR_EV)
    else:
        mat = Material(PERFECT, 0.0, 0.0)
    return Geom(R, L, ldim, mat, mat)


def logdetD(R, L, ldim, xi_, m, drude=None):
    g = geom(R, L, ldim, drude)
    return lib.oracle_logdetD(C.byref(g), float(xi_), int(m))


def logdetD_batch(R, L, ldim, xi_, m, drude=None, threads=1):
    g = geom(R, L, ldim, drude)
    xi_ = np.ascontiguousarray(xi_, dtype=np.float64)
    m = np.ascontiguousarray(m, dtype=np.int32)
    out = np.empty(len(xi_))
    lib.oracle_logdetD_batch(C.byref(g), len(xi_), xi_.ctypes.data_as(C.POINTER(C.c_double)),
                             m.ctypes.data_as(C.POINTER(C.c_int)), out.ctypes.data_as(C.POINTER(C.c_double)), threads)
    return out


def M_dense(R, L, ldim, xi_, m, drude=None):
    g = geom(R, L, ldim, drude)
    out = np.empty((2 * ldim, 2 * ldim))
    lib.oracle_M_dense(C.byref(g), float(xi_), int(m), out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def mie(LbyR, xi_, l, epsm1):
    a, b = C.c_double(), C.c_double()
    lib.oracle_mie(LbyR, xi_, l, epsm1, C.byref(a), C.byref(b))
    return a.value, b.value


def free_energy(R, L, ldim, T, drude=None, cutoff=1e-9, epsrel=1e-6, threads=1):
    g = geom(R, L, ldim, drude)
    xi = (C.c_double * 4096)()
    v = (C.c_double * 4096)()
    nxi, ndet = C.c_int(), C.c_int()
    E = lib.oracle_free_energy(C.byref(g), T, cutoff, epsrel, threads, xi, v, C.byref(nxi), C.byref(ndet))
    return E, dict(nxi=nxi.value, ndet=ndet.value, xi=list(xi[:nxi.value]), logdetD=list(v[:nxi.value]))


C_LIGHT = 299792458.0


def plasma_I(nu, omegap_):
    """I_nu of the plasma xi=0 block; omegap_ = omegap (L+R)/c"""
    return lib.oracle_plasma_I(int(nu), float(omegap_))


def logdetD0_MM_plasma(R, L, ldim, m, omegap_scaled):
    """omegap_scaled: plasma frequency in units of c/(L+R)"""
    g = geom(R, L, ldim)
    return lib.oracle_logdetD0_MM_plasma(C.byref(g), int(m), omegap_scaled * C_LIGHT / (L + R))


def ht_plasma(R, L, ldim, omegap_scaled, eps):
    g = geom(R, L, ldim)
    return lib.oracle_ht_plasma(C.byref(g), omegap_scaled * C_LIGHT / (L + R), float(eps))
