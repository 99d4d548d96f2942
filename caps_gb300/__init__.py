"""Python binding of the GB300 CaPS library (libcaps_gb300.so, C-ABI).

The binding mirrors the reference's C API (src/include/libcaps.h): a Caps
object wraps caps_t; logdetD, mie, M, logdetD0 and the batch/free-energy
extensions call straight into the CUDA library.  There is no CPU path: if the
shared library is missing, importing raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libcaps_gb300.so")

DETALG_HODLR, DETALG_LU, DETALG_QR, DETALG_CHOLESKY = 0, 1, 2, 3
PREC_FP64, PREC_MIXED = 0, 1
PATH_AUTO, PATH_HODLR, PATH_DENSE = 0, 1, 2
HBAR_EV = 6.582119514e-16
C_LIGHT = 299792458.0


def gauss_laguerre(n):
    """nodes x and weights w e^x of the n-point Gauss-Laguerre rule"""
    x, w = np.empty(n), np.empty(n)
    if not lib.caps_gauss_laguerre(int(n), x.ctypes.data_as(C.POINTER(C.c_double)), w.ctypes.data_as(C.POINTER(C.c_double))):
        raise ValueError("unsupported number of points")
    return x, w


class _AutotuneInfo(C.Structure):
    _fields_ = [("ncand", C.c_int), ("chosen", C.c_int), ("ms_per_matrix", C.c_double * 4)]


class _EnergyInfo(C.Structure):
    _fields_ = [("nxi", C.c_int), ("ndet", C.c_int), ("nwasted", C.c_int), ("seconds", C.c_double),
                ("xi", C.POINTER(C.c_double)), ("logdetD", C.POINTER(C.c_double))]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libcaps_gb300.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    d, i, vp, dp, ip = C.c_double, C.c_int, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int)
    sig = {
        "caps_init": (vp, [d, d]), "caps_free": (None, [vp]),
        "caps_set_ldim": (i, [vp, i]), "caps_get_ldim": (i, [vp]),
        "caps_set_detalg": (i, [vp, i]), "caps_get_detalg": (i, [vp]),
        "caps_set_epsrel": (i, [vp, d]), "caps_get_epsrel": (d, [vp]),
        "caps_set_epsilonm1": (None, [vp, vp, vp]),
        "material_init": (vp, [C.c_char_p, d]), "material_free": (None, [vp]),
        "material_epsilonm1": (d, [d, vp]), "material_get_extrapolation": (None, [vp, dp, dp, dp, dp]),
        "caps_set_epsilonm1_plate": (None, [vp, vp, vp]),
        "caps_set_epsilonm1_sphere": (None, [vp, vp, vp]),
        "caps_logdetD": (d, [vp, d, i]),
        "caps_logdetD_batch": (i, [vp, dp, ip, i, dp, ip]),
        "caps_mie": (None, [vp, d, i, dp, dp]), "caps_mie_perf": (None, [vp, d, i, dp, dp]),
        "caps_lnLambda": (d, [i, i, i]),
        "caps_fresnel": (None, [vp, d, d, dp, dp]),
        "caps_estimate_lminmax": (i, [vp, i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
        "caps_M_init": (vp, [vp, i, d]), "caps_M_elem": (d, [vp, i, i, C.c_char, C.c_char]),
        "caps_M_free": (None, [vp]), "caps_kernel_M": (d, [i, i, vp]),
        "caps_logdetD0": (None, [vp, i, d, dp, dp, dp]),
        "caps_ht_drude": (d, [vp]), "caps_ht_perf": (d, [vp, d]), "caps_ht_plasma": (d, [vp, d, d]),
        "caps_integrate_plasma_init": (vp, [vp, d, d]), "caps_integrate_plasma_free": (None, [vp]),
        "caps_integrate_plasma": (d, [vp, i, i, i, dp, dp]),
        "caps_free_energy": (d, [vp, d, d, d, C.POINTER(_EnergyInfo)]),
        "caps_free_energy_T0": (d, [vp, d, d, i, C.POINTER(_EnergyInfo)]),
        "caps_free_energy_T0_gl": (d, [vp, d, i, C.POINTER(_EnergyInfo)]),
        "caps_gauss_laguerre": (i, [i, dp, dp]),
        "caps_logdetD2_batch": (i, [vp, dp, ip, i, dp, ip]),
        "caps_sphere_sphere_T0": (d, [vp, d, d, C.POINTER(_EnergyInfo)]),
        "caps_free_energy_psd": (d, [vp, d, d, d, i, C.POINTER(_EnergyInfo)]),
        "caps_gpu_set_precision": (i, [vp, i]),
        "caps_gpu_set_path": (i, [vp, i]),
        "caps_gpu_autotune": (i, [vp, d, i, vp]),
        "caps_gpu_last_error": (C.c_char_p, []),
        "caps_gpu_set_stream": (None, [vp]),
        "caps_gpu_timings": (i, [dp, i]),
        "caps_gpu_reset_timings": (None, []),
        "caps_gpu_counters": (None, [C.POINTER(C.c_longlong)] * 3 + [i]),
        "caps_gpu_fp64_peak": (d, []),
        "caps_gpu_kernel_timing": (None, [i]),
        "caps_gpu_kernel_stats": (None, [dp, dp, C.POINTER(C.c_longlong)]),
        "caps_gpu_kernel_stats_kind": (None, [i, dp, dp, C.POINTER(C.c_longlong)]),
        "caps_gpu_fp32_peak": (d, []),
        "caps_gpu_work": (None, [C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), C.POINTER(C.c_double)]),
        "caps_logdetD_noalloc": (i, [vp, d, i, dp]),
        "caps_mlp_create": (vp, [C.c_uint]), "caps_mlp_free": (None, [vp]), "caps_mlp_nparams": (i, []),
        "caps_mlp_get_params": (None, [vp, C.POINTER(C.c_float)]), "caps_mlp_set_params": (None, [vp, C.POINTER(C.c_float)]),
        "caps_mlp_features": (None, [d, d, i, d, d, C.POINTER(C.c_float)]),
        "caps_mlp_loss_grad": (d, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), i, C.POINTER(C.c_float)]),
        "caps_mlp_train": (d, [vp, C.POINTER(C.c_float), C.POINTER(C.c_float), i, i, C.c_float]),
        "caps_mlp_predict": (None, [vp, C.POINTER(C.c_float), i, C.POINTER(C.c_float)]),
        "caps_mlp_proposal": (i, [vp, d, d, d, vp, i, ip]),
        "caps_free_energy_learned": (d, [vp, d, d, d, vp, C.POINTER(_EnergyInfo)]),
        "caps_noalloc_last_error": (C.c_char_p, []),
        "caps_capc_lmax": (i, [d, d, d]), "caps_capc_pfa": (d, [d, d]),
        "caps_capc_logdet": (d, [d, d, i, d, C.c_char, i]),
        "caps_capc_logdet_batch": (i, [d, d, i, dp, i, C.c_char, i, dp]),
        "caps_capc_energy_T0": (d, [d, d, i, C.c_char, d, i, ip, ip]),
        "bessel_logI0": (d, [d]), "bessel_logI1": (d, [d]), "bessel_logK0": (d, [d]), "bessel_logK1": (d, [d]),
        "bessel_logIn": (d, [i, d]), "bessel_logKn": (d, [i, d]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def last_error():
    return lib.caps_gpu_last_error().decode()


def set_stream(handle):
    """Run subsequent GPU work on the given cudaStream_t handle (int) or None."""
    lib.caps_gpu_set_stream(C.c_void_p(handle) if handle else None)


def kernel_timing(enable):
    """live CUDA-event timing of the factorisation's kernels on/off (resets the totals)"""
    lib.caps_gpu_kernel_timing(1 if enable else 0)


def kernel_stats(kind=0):
    """(device ms, algorithmic bytes, launches) since kernel_timing(True) of the tcgen05 trailing
    update (kind 0), the panel solve (1) or the diagonal block (2)"""
    ms, by, n = C.c_double(0), C.c_double(0), C.c_longlong(0)
    lib.caps_gpu_kernel_stats_kind(int(kind), C.byref(ms), C.byref(by), C.byref(n))
    return ms.value, by.value, n.value


def timings(cumulative=False):
    """device milliseconds per phase: setup+Mie, K, I, elements+stats, factorisation, total"""
    buf = (C.c_double * 12)()
    lib.caps_gpu_timings(buf, 12)
    return list(buf[6:12]) if cumulative else list(buf[:6])


def reset_timings():
    lib.caps_gpu_reset_timings()


def counters(reset=False):
    a, b, c = C.c_longlong(), C.c_longlong(), C.c_longlong()
    lib.caps_gpu_counters(C.byref(a), C.byref(b), C.byref(c), int(reset))
    return dict(launches=a.value, h2d=b.value, d2h=c.value)


def work():
    a, b, c = C.c_longlong(), C.c_longlong(), C.c_double()
    lib.caps_gpu_work(C.byref(a), C.byref(b), C.byref(c))
    return dict(nmat=a.value, nfactor=b.value, factor_flops=c.value)


def fp32_peak():
    return lib.caps_gpu_fp32_peak()


def fp64_peak():
    return lib.caps_gpu_fp64_peak()


class Caps:
    """caps_t of the reference API: R and L in metres."""

    def __init__(self, R, L, ldim=None, detalg=None):
        self._h = lib.caps_init(R, L)
        if not self._h:
            raise ValueError("caps_init failed (R and L must be positive)")
        self._ud = None
        self._mat = None
        self.R, self.L = R, L
        if ldim is not None:
            lib.caps_set_ldim(self._h, ldim)
        if detalg is not None:
            lib.caps_set_detalg(self._h, detalg)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.caps_free(h)
            self._h = None
        m = getattr(self, "_mat", None)
        if m:
            lib.material_free(m)
            self._mat = None

    def set_material(self, path):
        """plate and sphere from a tabulated optical-data file (material_init +
        material_epsilonm1, as the reference driver's --material)"""
        m = lib.material_init(os.fsencode(path), self.L + self.R)
        if not m:
            raise ValueError("material_init failed: %s (missing file or wrong format)" % path)
        fn = C.cast(lib.material_epsilonm1, C.c_void_p)
        lib.caps_set_epsilonm1(self._h, fn, m)
        if self._mat:
            lib.material_free(self._mat)
        self._mat = m

    @property
    def ldim(self):
        return lib.caps_get_ldim(self._h)

    def set_ldim(self, ldim):
        return lib.caps_set_ldim(self._h, ldim)

    def set_detalg(self, detalg):
        return lib.caps_set_detalg(self._h, detalg)

    def set_precision(self, prec):
        return lib.caps_gpu_set_precision(self._h, prec)

    def autotune(self, xi_, nprobe=8):
        """time the candidate schedules on nprobe matrices of this workload, keep the fastest;
        returns (chosen index, device ms per matrix of each candidate)"""
        info = _AutotuneInfo()
        lib.caps_gpu_autotune(self._h, float(xi_), int(nprobe), C.byref(info))
        return info.chosen, list(info.ms_per_matrix[:info.ncand])

    def set_path(self, path):
        """determinant path under DETALG_HODLR: PATH_AUTO, PATH_HODLR or PATH_DENSE"""
        return lib.caps_gpu_set_path(self._h, path)

    def set_drude(self, omegap_eV, gamma_eV):
        """Drude metal (gamma=0: plasma) for plate and sphere, via caps_epsilonm1_drude."""
        self._ud = (C.c_double * 2)(omegap_eV / HBAR_EV, gamma_eV / HBAR_EV)
        fn = C.cast(lib.caps_epsilonm1_drude, C.c_void_p)
        lib.caps_set_epsilonm1(self._h, fn, C.cast(self._ud, C.c_void_p))

    def logdetD(self, xi_, m):
        return lib.caps_logdetD(self._h, float(xi_), int(m))

    def logdetD_batch(self, xi_, m):
        xi_ = np.ascontiguousarray(xi_, dtype=np.float64)
        m = np.ascontiguousarray(m, dtype=np.int32)
        n = len(xi_)
        out = np.empty(n)
        st = np.empty(n, dtype=np.int32)
        lib.caps_logdetD_batch(self._h, xi_.ctypes.data_as(C.POINTER(C.c_double)), m.ctypes.data_as(C.POINTER(C.c_int)),
                               n, out.ctypes.data_as(C.POINTER(C.c_double)), st.ctypes.data_as(C.POINTER(C.c_int)))
        return out, st

    def mie(self, xi_, l):
        a, b = C.c_double(), C.c_double()
        lib.caps_mie(self._h, float(xi_), int(l), C.byref(a), C.byref(b))
        return a.value, b.value

    def mie_perf(self, xi_, l):
        a, b = C.c_double(), C.c_double()
        lib.caps_mie_perf(self._h, float(xi_), int(l), C.byref(a), C.byref(b))
        return a.value, b.value

    def lminmax(self, m):
        lo, hi = C.c_size_t(), C.c_size_t()
        lib.caps_estimate_lminmax(self._h, int(m), C.byref(lo), C.byref(hi))
        return lo.value, hi.value

    def fresnel(self, xi_, k_):
        a, b = C.c_double(), C.c_double()
        lib.caps_fresnel(self._h, float(xi_), float(k_), C.byref(a), C.byref(b))
        return a.value, b.value

    def M(self, xi_, m):
        """Dense round-trip matrix (2 ldim x 2 ldim, interleaved E/M) via caps_M_init."""
        h = lib.caps_M_init(self._h, int(m), float(xi_))
        dim = 2 * self.ldim
        out = np.empty((dim, dim))
        for i in range(dim):
            for j in range(dim):
                out[i, j] = lib.caps_kernel_M(i, j, h)
        lib.caps_M_free(h)
        return out

    def logdetD0(self, m, EE=True, MM=True):
        ee, mm = C.c_double(np.nan), C.c_double(np.nan)
        lib.caps_logdetD0(self._h, int(m), 0.0, C.byref(ee) if EE else None, C.byref(mm) if MM else None, None)
        return ee.value, mm.value

    def logdetD0_plasma(self, m, omegap):
        """xi=0 MM block of the plasma model; omegap in rad/s"""
        v = C.c_double(np.nan)
        lib.caps_logdetD0(self._h, int(m), float(omegap), None, None, C.byref(v))
        return v.value

    def ht_plasma(self, omegap, eps):
        """high-temperature free energy of the plasma model (units of kB T); omegap in rad/s"""
        return lib.caps_ht_plasma(self._h, float(omegap), float(eps))

    def integrate_plasma(self, omegap, pairs):
        """[(I, ratio1, ratio2)] of caps_integrate_plasma for (l1, l2, m) triples"""
        h = lib.caps_integrate_plasma_init(self._h, float(omegap), 1e-8)
        try:
            out = []
            for l1, l2, m in pairs:
                r1, r2 = C.c_double(), C.c_double()
                v = lib.caps_integrate_plasma(h, int(l1), int(l2), int(m), C.byref(r1), C.byref(r2))
                out.append((v, r1.value, r2.value))
            return out
        finally:
            lib.caps_integrate_plasma_free(h)

    def ht_drude(self):
        return lib.caps_ht_drude(self._h)

    def ht_perf(self, eps):
        return lib.caps_ht_perf(self._h, eps)

    def free_energy(self, T, cutoff=1e-9, epsrel=1e-6, mlp=None):
        """free energy E (L+R)/(hbar c); with mlp (an MLP) the learned proposal sizes the batch"""
        xi = (C.c_double * 4096)()
        v = (C.c_double * 4096)()
        info = _EnergyInfo(0, 0, 0, 0.0, C.cast(xi, C.POINTER(C.c_double)), C.cast(v, C.POINTER(C.c_double)))
        if mlp is not None:
            E = lib.caps_free_energy_learned(self._h, float(T), float(cutoff), float(epsrel), mlp._h, C.byref(info))
        else:
            E = lib.caps_free_energy(self._h, float(T), float(cutoff), float(epsrel), C.byref(info))
        n = info.nxi
        return E, dict(nxi=n, ndet=info.ndet, nwasted=info.nwasted, seconds=info.seconds,
                       xi=list(xi[:n]), logdetD=list(v[:n]))

    def _energy(self, call):
        xi = (C.c_double * 4096)()
        v = (C.c_double * 4096)()
        info = _EnergyInfo(0, 0, 0, 0.0, C.cast(xi, C.POINTER(C.c_double)), C.cast(v, C.POINTER(C.c_double)))
        E = call(C.byref(info))
        n = min(info.nxi, 4096)
        return E, dict(nxi=info.nxi, ndet=info.ndet, nwasted=info.nwasted, seconds=info.seconds,
                       xi=list(xi[:n]), logdetD=list(v[:n]))

    def free_energy_T0(self, cutoff=1e-9, epsrel=1e-6, method="qagi"):
        """free energy at T = 0, E (L+R)/(hbar c); method "qagi" (the reference's default) or "fcqs"."""
        m = {"qagi": 0, "fcqs": 1}[method]
        return self._energy(lambda info: lib.caps_free_energy_T0(self._h, float(cutoff), float(epsrel), m, info))

    def free_energy_T0_gl(self, n=60, cutoff=1e-9):
        """free energy at T = 0 by an n-point Gauss-Laguerre rule in x = 2 xi L/c"""
        return self._energy(lambda info: lib.caps_free_energy_T0_gl(self._h, float(cutoff), int(n), info))

    def logdetD2_batch(self, xi_, m):
        """sphere-sphere: log det(1 - M^2) per (xi, m); make the object with L = d/2"""
        xi_ = np.ascontiguousarray(xi_, dtype=np.float64)
        m = np.ascontiguousarray(m, dtype=np.int32)
        n = len(xi_)
        out = np.empty(n)
        st = np.empty(n, dtype=np.int32)
        lib.caps_logdetD2_batch(self._h, xi_.ctypes.data_as(C.POINTER(C.c_double)), m.ctypes.data_as(C.POINTER(C.c_int)), n,
                                out.ctypes.data_as(C.POINTER(C.c_double)), st.ctypes.data_as(C.POINTER(C.c_int)))
        return out, st

    def sphere_sphere_T0(self, cutoff=1e-10, epsrel=1e-6):
        """two spheres of radius R at separation d = 2L, T = 0: E d/(hbar c)"""
        return self._energy(lambda info: lib.caps_sphere_sphere_T0(self._h, float(cutoff), float(epsrel), info))

    def free_energy_psd(self, T, cutoff=1e-9, epsrel=1e-6, order=0):
        """free energy at T > 0 by Pade spectrum decomposition (order <= 0: automatic)"""
        return self._energy(lambda info: lib.caps_free_energy_psd(self._h, float(T), float(cutoff), float(epsrel), int(order), info))


class MLP:
    """the learned-truncation network (caps_mlp_t): 5-64-64-64-1 SiLU, trained on the GPU"""

    def __init__(self, seed=0):
        self._h = lib.caps_mlp_create(seed)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.caps_mlp_free(h)
            self._h = None

    @staticmethod
    def nparams():
        return lib.caps_mlp_nparams()

    def params(self):
        out = np.empty(self.nparams(), dtype=np.float32)
        lib.caps_mlp_get_params(self._h, out.ctypes.data_as(C.POINTER(C.c_float)))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        lib.caps_mlp_set_params(self._h, p.ctypes.data_as(C.POINTER(C.c_float)))

    @staticmethod
    def features(RbyL, xi_, m, omegap_eV, gamma_eV):
        x = (C.c_float * 5)()
        lib.caps_mlp_features(RbyL, xi_, m, omegap_eV, gamma_eV, x)
        return np.array(x[:], dtype=np.float32)

    def loss_grad(self, X, y):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(self.nparams(), dtype=np.float32)
        loss = lib.caps_mlp_loss_grad(self._h, X.ctypes.data_as(C.POINTER(C.c_float)), y.ctypes.data_as(C.POINTER(C.c_float)),
                                      len(y), g.ctypes.data_as(C.POINTER(C.c_float)))
        return loss, g

    def train(self, X, y, epochs=2000, lr=3e-3):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        return lib.caps_mlp_train(self._h, X.ctypes.data_as(C.POINTER(C.c_float)), y.ctypes.data_as(C.POINTER(C.c_float)),
                                  len(y), epochs, lr)

    def predict(self, X):
        X = np.ascontiguousarray(X, dtype=np.float32)
        y = np.empty(len(X), dtype=np.float32)
        lib.caps_mlp_predict(self._h, X.ctypes.data_as(C.POINTER(C.c_float)), len(X), y.ctypes.data_as(C.POINTER(C.c_float)))
        return y

    def proposal(self, caps, T, cutoff=1e-9, epsrel=1e-6, nmax=256):
        ch = np.zeros(nmax, dtype=np.int32)
        N = lib.caps_mlp_proposal(caps._h, float(T), float(cutoff), float(epsrel), self._h, nmax,
                                  ch.ctypes.data_as(C.POINTER(C.c_int)))
        return N, ch[:max(N, 0)]


# ---- cylinder-plane geometry (the reference's capc program) ----

_DETALG = {"HODLR": 0, "LU": 1, "QR": 2, "CHOLESKY": 3}


def capc_lmax(R, d, eta=6.0):
    """the capc program's dimension max(25, ceil(eta R/d))"""
    return lib.caps_capc_lmax(float(R), float(d), float(eta))


def capc_logdet(R, d, q, DN="D", lmax=0, detalg="HODLR"):
    """CasimirCP::logdet for one wave number q or an array of them (one GPU batch)"""
    qs = np.atleast_1d(np.ascontiguousarray(q, dtype=np.float64))
    out = np.empty_like(qs)
    lib.caps_capc_logdet_batch(float(R), float(d), int(lmax), qs.ctypes.data_as(C.POINTER(C.c_double)), len(qs),
                               DN.encode()[:1], _DETALG[detalg.upper()], out.ctypes.data_as(C.POINTER(C.c_double)))
    return out if np.ndim(q) else float(out[0])


def capc_energy_T0(R, d, p="D", lmax=0, epsrel=1e-8, detalg="HODLR"):
    """CasimirCP::energy at T = 0: (E/(hbar c L), qagi neval, qagi ier)"""
    ne, ier = C.c_int(0), C.c_int(0)
    E = lib.caps_capc_energy_T0(float(R), float(d), int(lmax), p.encode()[:1], float(epsrel), _DETALG[detalg.upper()],
                                C.byref(ne), C.byref(ier))
    return E, ne.value, ier.value
