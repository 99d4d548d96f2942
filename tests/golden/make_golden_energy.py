"""Golden free energies from the unmodified reference library (oracle/_ref).

Restates the serial master loop of the caps driver (src/caps.c:307-396 F_xi,
:749-852 Matsubara sum) in Python around caps_logdetD of libcaps_ref.so, with
the m loop farmed out to a process pool (results are summed in m order, so the
value does not depend on the pool size).  Writes tests/golden/energy_<name>.json.

    python tests/golden/make_golden_energy.py c3      # Drude, R/L=150 (~30 CPU-min)
    python tests/golden/make_golden_energy.py small   # PR and Drude, R/L=10
    python tests/golden/make_golden_energy.py plasma  # plasma model (gamma = 0), R/L=10
    python tests/golden/make_golden_energy.py t0      # T = 0 (reference dqagi), Drude, R/L=20
    python tests/golden/make_golden_energy.py psd     # Pade spectrum decomposition, Drude, R/L=10
    python tests/golden/make_golden_energy.py material  # tabulated material (tests/golden/material_synthetic.txt)
"""
import ctypes as C
import json
import math
import multiprocessing as mp
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "libcaps_ref.so")
HBAR, HBAR_EV, KB, CL = 1.0545718e-34, 6.582119514e-16, 1.38064852e-23, 299792458.0
_lib = None


def _init():
    global _lib
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    _lib = C.CDLL(REF)
    _lib.caps_init.restype = C.c_void_p
    _lib.caps_init.argtypes = [C.c_double, C.c_double]
    _lib.caps_logdetD.restype = C.c_double
    _lib.caps_logdetD.argtypes = [C.c_void_p, C.c_double, C.c_int]
    _lib.caps_set_ldim.argtypes = [C.c_void_p, C.c_int]
    _lib.caps_set_detalg.argtypes = [C.c_void_p, C.c_int]
    _lib.caps_set_epsilonm1.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
    _lib.caps_free.argtypes = [C.c_void_p]
    _lib.caps_ht_drude.restype = C.c_double
    _lib.caps_ht_drude.argtypes = [C.c_void_p]
    _lib.caps_logdetD0.argtypes = [C.c_void_p, C.c_int, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    _lib.material_init.restype = C.c_void_p
    _lib.material_init.argtypes = [C.c_char_p, C.c_double]
    _lib.material_free.argtypes = [C.c_void_p]


def _task(args):
    R, L, ldim, drude, xi, m, detalg = args
    c = _lib.caps_init(R, L)
    _lib.caps_set_ldim(c, ldim)
    _lib.caps_set_detalg(c, detalg)
    ud = None
    mat = None
    if isinstance(drude, str):
        # tabulated material (the caps driver's --material, caps.c:573-586)
        mat = _lib.material_init(os.path.join(ROOT, drude).encode(), R + L)
        _lib.caps_set_epsilonm1(c, C.cast(_lib.material_epsilonm1, C.c_void_p), C.c_void_p(mat))
    elif drude:
        ud = (C.c_double * 2)(drude[0] / HBAR_EV, drude[1] / HBAR_EV)
        _lib.caps_set_epsilonm1(c, C.cast(_lib.caps_epsilonm1_drude, C.c_void_p), C.cast(ud, C.c_void_p))
    if xi == 0 and drude:
        # plasma model (gamma = 0): the MM_plasma block (caps.c:927-929)
        v = C.c_double()
        _lib.caps_logdetD0(c, m, drude[0] / HBAR_EV, None, None, C.byref(v))
        r = v.value
    elif xi == 0:
        v = C.c_double()
        _lib.caps_logdetD0(c, m, 0.0, None, C.byref(v), None)
        r = v.value
    else:
        r = _lib.caps_logdetD(c, xi, m)
    _lib.caps_free(c)
    if mat:
        _lib.material_free(mat)
    return r


def kahan(v):
    s = c = 0.0
    for x in v:
        y = x - c
        t = s + y
        c = (t - s) - y
        s = t
    return s


def F_xi(pool, R, L, ldim, drude, xi, cutoff, detalg, chunk):
    terms, m0 = [], 0
    while True:
        vals = pool.map(_task, [(R, L, ldim, drude, xi, m, detalg) for m in range(m0, m0 + chunk)])
        for v in vals:
            terms.append(v)
            if v == 0 or v / terms[0] < cutoff:
                t = terms[:]
                t[0] /= 2
                return kahan(t), len(terms), terms
        m0 += chunk


def energy(R, L, ldim, T, drude, cutoff=1e-9, epsrel=1e-6, detalg=1, procs=8):
    Ts = 2 * math.pi * KB * (R + L) * T / (HBAR * CL)
    _init()
    with mp.Pool(procs, initializer=_init) as pool:
        c = _lib.caps_init(R, L)
        _lib.caps_set_ldim(c, ldim)
        if isinstance(drude, str) or (drude and drude[1] > 0):
            # Drude, or a material whose low-frequency extrapolation is Drude (gamma_low > 0)
            v0 = _lib.caps_ht_drude(c)
        else:
            # perfect reflectors and the plasma model (caps.c:329-395)
            drude_ht = _lib.caps_ht_drude(c)
            s, _, _ = F_xi(pool, R, L, ldim, drude, 0.0, cutoff, detalg, procs)
            v0 = drude_ht + s
        v, xis, ndet, per_m = [v0], [0.0], 0, []
        n = 1
        while True:
            s, nm, terms = F_xi(pool, R, L, ldim, drude, n * Ts, cutoff, detalg, procs)
            ndet += nm
            v.append(s)
            xis.append(n * Ts)
            per_m.append(terms)
            print("n=%d xi=%.16g v=%.16g m=%d" % (n, n * Ts, s, nm), file=sys.stderr, flush=True)
            if abs(s / v[0]) < epsrel:
                break
            n += 1
    w = v[:]
    w[0] /= 2
    # terms[k][m]: the reference's logdetD(xi_{k+1}, m) for every m its cutoff visits
    return Ts / math.pi * kahan(w), dict(xi=xis, logdetD=v, ndet=ndet, terms=per_m)


def energy_t0(R, L, ldim, drude, cutoff=1e-9, epsrel=1e-6, detalg=1, procs=8):
    """T = 0 (caps.c:722-748): the reference's dqagi over x = 2 xi L/c of F(x/alpha), with
    the PFA cut of the integrand (caps.c:235-267)"""
    alpha = 2 * L / (L + R)
    LbyR = L / R
    xi_cutoff = -(1 + 1 / LbyR) * math.log(2 * LbyR * 1e-100) / 2
    _init()
    FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)
    _lib.dqagi.restype = C.c_double
    _lib.dqagi.argtypes = [FN, C.c_double, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int),
                           C.POINTER(C.c_int), C.c_void_p]
    xis, vals, ndet = [], [], [0]
    with mp.Pool(procs, initializer=_init) as pool:
        def integrand(x, _u):
            xi = x / alpha
            if LbyR < 0.1 and xi > xi_cutoff:
                v = 0.0
            else:
                v, nm, _ = F_xi(pool, R, L, ldim, drude, xi, cutoff, detalg, procs)
                ndet[0] += nm
            xis.append(xi)
            vals.append(v)
            return v
        cb = FN(integrand)
        ab, ne, ier = C.c_double(), C.c_int(), C.c_int()
        r = _lib.dqagi(cb, 0.0, 1, 0.0, epsrel, C.byref(ab), C.byref(ne), C.byref(ier), None)
    return r / alpha / math.pi, dict(xi=xis, logdetD=vals, ndet=ndet[0], neval=ne.value, ier=ier.value, abserr=ab.value)


def energy_psd(R, L, ldim, T, drude, cutoff=1e-9, epsrel=1e-6, detalg=1, procs=8):
    """T > 0 by Pade spectrum decomposition (caps.c:635-639, 811-831) with the reference's
    psd() poles and weights"""
    Ts = 2 * math.pi * KB * (R + L) * T / (HBAR * CL)
    Teff = 4 * math.pi * KB / HBAR / CL * T * L
    order = int(math.ceil((1 - 1.5 * math.log10(epsrel)) / math.sqrt(Teff)))
    _init()
    _lib.psd.restype = C.c_int
    _lib.psd.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    pxi, peta = (C.c_double * order)(), (C.c_double * order)()
    assert _lib.psd(order, pxi, peta) == 0
    with mp.Pool(procs, initializer=_init) as pool:
        c = _lib.caps_init(R, L)
        _lib.caps_set_ldim(c, ldim)
        if drude and drude[1] > 0:
            v0 = _lib.caps_ht_drude(c)
        else:
            s, _, _ = F_xi(pool, R, L, ldim, drude, 0.0, cutoff, detalg, procs)
            v0 = _lib.caps_ht_drude(c) + s
        v, xis, ndet = [v0], [0.0], 0
        for n in range(order):
            xi = pxi[n] * Ts / (2 * math.pi)
            s, nm, _ = F_xi(pool, R, L, ldim, drude, xi, cutoff, detalg, procs)
            ndet += nm
            v.append(peta[n] * s)
            xis.append(xi)
    w = v[:]
    w[0] /= 2
    return Ts / math.pi * kahan(w), dict(xi=xis, logdetD=v, ndet=ndet, order=order)


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "small"
    procs = int(os.environ.get("PROCS", "8"))
    cases = {
        "small": [("pr_RbyL10_ldim70_T300", 10e-6, 1e-6, 70, 300.0, None), ("drude_RbyL10_ldim70_T300", 10e-6, 1e-6, 70, 300.0, (9.0, 0.035))],
        "plasma": [("plasma_RbyL10_ldim70_T300", 10e-6, 1e-6, 70, 300.0, (9.0, 0.0))],
        "material": [("material_RbyL10_ldim70_T300", 10e-6, 1e-6, 70, 300.0, "tests/golden/material_synthetic.txt")],
        "t0": [("t0_drude_RbyL20_ldim100", 20e-6, 1e-6, 100, 0.0, (9.0, 0.035))],
        "psd": [("psd_drude_RbyL10_ldim70_T300", 10e-6, 1e-6, 70, 300.0, (9.0, 0.035))],
        "c2": [("pr_RbyL50_ldim350_T300", 50e-6, 1e-6, 350, 300.0, None)],
        "c3": [("drude_RbyL150_ldim1050_T300", 150e-6, 1e-6, 1050, 300.0, (9.0, 0.035))],
    }[which]
    for name, R, L, ldim, T, drude in cases:
        t = time.time()
        if which == "t0":
            E, info = energy_t0(R, L, ldim, drude, procs=procs)
        elif which == "psd":
            E, info = energy_psd(R, L, ldim, T, drude, procs=procs)
        else:
            E, info = energy(R, L, ldim, T, drude, procs=procs)
        info.update(R=R, L=L, ldim=ldim, T=T, drude=drude, E=E, cutoff=1e-9, epsrel=1e-6, detalg="LU",
                    seconds=time.time() - t, procs=procs, source="oracle/_ref/libcaps_ref.so via tests/golden/make_golden_energy.py")
        json.dump(info, open(os.path.join(HERE, "energy_%s.json" % name), "w"), indent=1)
        print(name, E, info["ndet"], time.time() - t, file=sys.stderr)
