"""Generate the golden fixtures of tests/golden/ from the CaPS v0.5 reference.

Run here, where the reference source tree and its build (oracle/_ref, made by
oracle/Makefile.ref) exist:

    CAPS_REFERENCE_SRC=<CaPS source tree> python tests/golden/make_golden.py [--heavy]

Two sources:
 1. known-answer vectors of the reference's own unit tests, read as text from
    src/tests/test_logdetD.c, test_mie.c and test_mie_drude.c;
 2. values computed by the unmodified reference library (libcaps_ref.so):
    logdetD per (xi,m) for the benchmark geometries (LU and HODLR), Mie
    coefficients, K and I integrals, and dense round-trip matrices.
The machines that run the tests need no reference tree: the tests read only the JSON written here.
"""
import argparse
import ctypes as C
import json
import os
import re
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HBAR_EV = 6.582119514e-16
CLIGHT = 299792458.0


def _read_c(path):
    """source text without /* */ comments (the reference disables some vectors that way)"""
    return re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)


def parse_tests(ref):
    out = {}
    t = _read_c(os.path.join(ref, "src/tests/test_logdetD.c"))
    body = t[t.index("int test_logdetD()"):t.index("int test_logdetD0()")]
    arrays = {}
    for name, vals in re.findall(r"double (v\d)\[\] = \{(.*?)\};", body, re.S):
        arrays[name] = [float(x) for x in re.findall(r"(-?\d+\.\d+(?:e-?\d+)?)", vals)]
    cases = []
    for m, v in enumerate(arrays["v1"]):
        cases.append(dict(R=1.0, L=0.01, ldim=500, xi=1.0, m=m, logdetD=v))
    for m, v in enumerate(arrays["v2"]):
        cases.append(dict(R=1.0, L=0.01, ldim=500, xi=0.1, m=m, logdetD=v))
    for m, v in enumerate(arrays["v3"]):
        cases.append(dict(R=1.0, L=0.01, ldim=500, xi=10.0, m=m, logdetD=v))
    big = body[body.index("caps_init(1,0.001)"):]
    for xi, m, v in re.findall(r"caps_logdetD\(caps, ([\d.]+),\s*(\d+)\), (-?[\d.e-]+)\)", big):
        cases.append(dict(R=1.0, L=0.001, ldim=10000, xi=float(xi), m=int(m), logdetD=float(v)))
    out["test_logdetD"] = dict(source="src/tests/test_logdetD.c:13-102", tolerance=1e-10, detalg="HODLR", cases=cases)

    body0 = t[t.index("int test_logdetD0()"):]
    eps = float(re.search(r"const double eps = ([\d.e-]+);", body0).group(1))
    cases = []
    for wp, v in re.findall(r"caps_ht_plasma\(caps,\s*([\d.]+)\*CAPS_c/\(L\+R\), eps\), (-?[\d.]+)\)", body0):
        cases.append(dict(R=100e-6, L=1e-6, ldim=500, omegap_scaled=float(wp), eps=eps, ht_plasma=float(v)))
    an = re.search(r"caps_logdetD0\(caps, 0, INFINITY, &EE, &MM, NULL\);\s*AssertAlmostEqual\(&test, EE, (-?[\d.]+)\);"
                   r"\s*AssertAlmostEqual\(&test, MM, (-?[\d.]+)\);", body0)
    out["test_logdetD0"] = dict(source="src/tests/test_logdetD.c:108-142", tolerance=1e-10, detalg="HODLR",
                                note="omegap in units of c/(L+R)", ht_plasma=cases,
                                m0_RbyL1000=dict(R=1.0, L=0.001, ldim=12000, m=0, EE=float(an.group(1)), MM=float(an.group(2))))

    t = _read_c(os.path.join(ref, "src/tests/test_fresnel.c"))
    R, L = (float(x) for x in re.search(r"caps_init\(([\d.e+-]+),([\d.e+-]+)\)", t).groups())
    cases = []
    for blk in re.split(r"userdata\[0\] = ", t)[1:]:
        wp = float(re.match(r"([\d.e+-]+)/CAPS_hbar_eV", blk).group(1))
        ga = float(re.search(r"userdata\[1\] = ([\d.e+-]+)/CAPS_hbar_eV", blk).group(1))
        for xi, k, te, tm in re.findall(r"caps_fresnel\(caps, ([\d.e+-]+), ([\d.e+-]+), &rTE, &rTM\);\s*"
                                        r"AssertAlmostEqual\(&test, rTE, (-?[\d.e+-]+)\);\s*"
                                        r"AssertAlmostEqual\(&test, rTM, (-?[\d.e+-]+)\);", blk):
            cases.append(dict(omegap_eV=wp, gamma_eV=ga, xi=float(xi), k=float(k), rTE=float(te), rTM=float(tm)))
    out["test_fresnel"] = dict(source="src/tests/test_fresnel.c:10-7025", tolerance=2e-15, R=R, L=L,
                               note="Drude epsilon-1 with omega_p, gamma in eV (userdata = value/hbar_eV)", cases=cases)

    t = _read_c(os.path.join(ref, "src/tests/test_mie.c"))
    cases = []
    for xi, l, blk in re.findall(r"caps_mie_perf\(self, ([\d.]+), (\d+), &lna, &lnb\);(.*?)(?=caps_mie_perf|caps_free)", t, re.S):
        vals = re.findall(r"AssertAlmostEqual\(&test, (ln[ab]), (-?[\d.]+(?:e-?\d+)?)\)", blk)
        d = dict(LbyR=1.0, xi=float(xi), l=int(l))
        for k, v in vals:
            d[k] = float(v)
        cases.append(d)
    out["test_mie_perf"] = dict(source="src/tests/test_mie.c:11-174", tolerance=1e-14, cases=cases)

    t = _read_c(os.path.join(ref, "src/tests/test_mie_drude.c"))
    cases = []
    parts = re.split(r"userdata\[0\] = ", t)[1:]
    for blk in parts:
        ud = re.match(r"([\d.]+)\*CAPS_c/\(L\+R\); userdata\[1\] = ([\d.]*)\*?CAPS_c/\(L\+R\);", blk)
        if not ud:
            continue
        wp = float(ud.group(1))
        gam = float(ud.group(2)) if ud.group(2) else 1.0
        for xi, l, rest in re.findall(r"caps_mie\(caps, ([\d.e-]+), (\d+), &lna, &lnb\);(.*?)(?=caps_mie\(|caps_free|userdata)", blk, re.S):
            vals = re.findall(r"AssertAlmostEqual\(&test, (ln[ab]), (-?[\d.]+(?:e-?\d+)?)\)", rest)
            d = dict(R=100e-6, L=100e-6, omegap_scaled=wp, gamma_scaled=gam, xi=float(xi), l=int(l))
            for k, v in vals:
                d[k] = float(v)
            cases.append(d)
    out["test_mie_drude"] = dict(source="src/tests/test_mie_drude.c:13-", tolerance=1e-11,
                                 note="omegap and gamma in units of c/(L+R)", cases=cases)
    return out


class Ref:
    def __init__(self, path):
        self.lib = lib = C.CDLL(path)
        lib.caps_init.restype = C.c_void_p
        lib.caps_init.argtypes = [C.c_double, C.c_double]
        lib.caps_logdetD.restype = C.c_double
        lib.caps_logdetD.argtypes = [C.c_void_p, C.c_double, C.c_int]
        for f in ("caps_set_ldim", "caps_set_detalg"):
            getattr(lib, f).argtypes = [C.c_void_p, C.c_int]
        lib.caps_set_epsilonm1.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.caps_free.argtypes = [C.c_void_p]
        lib.caps_mie.argtypes = [C.c_void_p, C.c_double, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        lib.caps_M_init.restype = C.c_void_p
        lib.caps_M_init.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.caps_kernel_M.restype = C.c_double
        lib.caps_kernel_M.argtypes = [C.c_int, C.c_int, C.c_void_p]
        lib.caps_M_free.argtypes = [C.c_void_p]
        lib.caps_integrate_init.restype = C.c_void_p
        lib.caps_integrate_init.argtypes = [C.c_void_p, C.c_double, C.c_int, C.c_double]
        lib.caps_integrate_K.restype = C.c_double
        lib.caps_integrate_K.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_byte)]
        lib.caps_integrate_I.restype = C.c_double
        lib.caps_integrate_I.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_byte)]
        lib.caps_integrate_free.argtypes = [C.c_void_p]
        self._keep = []

    def caps(self, R, L, ldim, drude=None, detalg=1):
        c = self.lib.caps_init(R, L)
        self.lib.caps_set_ldim(c, ldim)
        self.lib.caps_set_detalg(c, detalg)
        if drude:
            ud = (C.c_double * 2)(drude[0] / HBAR_EV, drude[1] / HBAR_EV)
            self._keep.append(ud)
            self.lib.caps_set_epsilonm1(c, C.cast(self.lib.caps_epsilonm1_drude, C.c_void_p), C.cast(ud, C.c_void_p))
        return c


def reference_values(ref_lib, heavy):
    r = Ref(ref_lib)
    out = {}
    # logdetD for the benchmark geometries and a spread of (xi, m)
    sets = [
        ("pr_RbyL20_ldim140", 20e-6, 1e-6, 140, None, [(1.0, m) for m in (0, 1, 2, 5, 10, 20, 34)] + [(0.1, 3), (7.5, 2), (41.5, 0)]),
        ("drude_RbyL20_ldim140", 20e-6, 1e-6, 140, (9.0, 0.035), [(0.5, 0), (1.0, 1), (3.0, 2), (12.0, 7), (60.0, 3)]),
        ("pr_RbyL50_ldim350", 50e-6, 1e-6, 350, None, [(41.98146, 0), (41.98146, 3), (83.96292, 10), (41.98146, 60)]),
        ("drude_RbyL150_ldim80", 150e-6, 1e-6, 80, (9.0, 0.035), [(124.298, 0), (124.298, 50), (248.596, 100)]),
    ]
    if heavy:
        sets.append(("drude_RbyL150_ldim1050", 150e-6, 1e-6, 1050, (9.0, 0.035), [(124.2980585533627, 10), (372.894175660088, 40), (124.2980585533627, 150)]))
    for name, R, L, ldim, drude, pts in sets:
        cases = []
        for xi, m in pts:
            row = dict(R=R, L=L, ldim=ldim, xi=xi, m=m, drude=drude)
            for alg, key in ((1, "LU"), (0, "HODLR")):
                c = r.caps(R, L, ldim, drude, detalg=alg)
                t = time.time()
                row[key] = r.lib.caps_logdetD(c, xi, m)
                row[key + "_seconds"] = time.time() - t
                r.lib.caps_free(c)
            cases.append(row)
            print(name, xi, m, row["LU"], row["HODLR"], file=sys.stderr)
        out[name] = cases
    # dense matrices M (reference element API) for element-level parity
    mats = []
    for R, L, ldim, drude, xi, m in [(20e-6, 1e-6, 24, None, 1.0, 0), (20e-6, 1e-6, 24, None, 1.0, 3),
                                     (20e-6, 1e-6, 24, (9.0, 0.035), 2.0, 2), (150e-6, 1e-6, 16, (9.0, 0.035), 124.298, 40)]:
        c = r.caps(R, L, ldim, drude)
        h = r.lib.caps_M_init(c, m, xi)
        n = 2 * ldim
        M = [[r.lib.caps_kernel_M(i, j, h) for j in range(n)] for i in range(n)]
        r.lib.caps_M_free(h)
        r.lib.caps_free(c)
        mats.append(dict(R=R, L=L, ldim=ldim, drude=drude, xi=xi, m=m, M=M))
    out["dense_M"] = mats
    # K and I integrals (log|.|, sign) from the reference integration object
    kis = []
    for R, L, ldim, drude, xi, m in [(20e-6, 1e-6, 140, None, 1.0, 0), (20e-6, 1e-6, 140, (9.0, 0.035), 3.0, 2),
                                     (150e-6, 1e-6, 1050, (9.0, 0.035), 124.298, 10)]:
        c = r.caps(R, L, ldim, drude)
        integ = r.lib.caps_integrate_init(c, xi, m, 1e-8)
        s = C.c_byte()
        mu = 2 * max(m, 1)
        lmin = 1 if m == 0 else max(m, int(round(m / np.sqrt(2 * L / R))) - ldim // 2)
        nus = sorted(set(list(range(mu, mu + 6)) + list(range(mu, 2 * (lmin + ldim) + 1, max(1, (2 * ldim) // 13)))))
        K = {}
        for p in (0, 1):
            K[p] = [(nu, r.lib.caps_integrate_K(integ, nu, p, C.byref(s)), int(s.value)) for nu in nus]
        ls = sorted(set([lmin, lmin + 1, lmin + ldim // 3, lmin + ldim // 2, lmin + ldim - 1]))
        I = []
        for l1 in ls:
            for l2 in ls:
                for p in (0, 1):
                    v = r.lib.caps_integrate_I(integ, l1, l2, p, C.byref(s))
                    I.append((l1, l2, p, v, int(s.value)))
        r.lib.caps_integrate_free(integ)
        r.lib.caps_free(c)
        kis.append(dict(R=R, L=L, ldim=ldim, drude=drude, xi=xi, m=m, K_TE=K[0], K_TM=K[1], I=I))
    out["K_I"] = kis
    # Mie coefficients on a grid (Drude, benchmark material)
    mie = []
    for R, L, drude in [(20e-6, 1e-6, None), (150e-6, 1e-6, (9.0, 0.035))]:
        c = r.caps(R, L, 100, drude)
        for xi in (0.05, 1.0, 124.298, 1118.68):
            for l in (1, 2, 10, 99, 100, 101, 500, 2000):
                a, b = C.c_double(), C.c_double()
                r.lib.caps_mie(c, xi, l, C.byref(a), C.byref(b))
                mie.append(dict(R=R, L=L, drude=drude, xi=xi, l=l, lna=a.value, lnb=b.value))
        r.lib.caps_free(c)
    out["mie_grid"] = mie
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CAPS_REFERENCE_SRC"),
                    help="CaPS source tree (default: $CAPS_REFERENCE_SRC)")
    ap.add_argument("--heavy", action="store_true")
    ap.add_argument("--unit-tests-only", action="store_true", help="re-parse the unit-test vectors only")
    a = ap.parse_args()
    if not a.ref:
        ap.error("set CAPS_REFERENCE_SRC (or --ref) to the CaPS source tree")
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    g = parse_tests(a.ref)
    json.dump(g, open(os.path.join(HERE, "reference_unit_tests.json"), "w"), indent=1)
    if a.unit_tests_only:
        print({k: len(x.get("cases", [])) for k, x in g.items()})
        return
    lib = os.path.join(ROOT, "oracle", "_ref", "libcaps_ref.so")
    v = reference_values(lib, a.heavy)
    json.dump(v, open(os.path.join(HERE, "reference_values.json"), "w"), indent=1)
    print({k: len(x["cases"]) for k, x in g.items()}, {k: len(x) for k, x in v.items()})


if __name__ == "__main__":
    main()
