"""Golden results of the reference's own quadratures and PSD poles, from the unmodified
reference library built here (oracle/_ref/libcaps_ref.so): dqagi (cquadpack), fcqs_semiinf
(src/fcqs.c) and psd (src/psd.c) on the integrands of tests/quad_cases.py.

    python tests/golden/make_golden_quad.py      # writes tests/golden/quad_golden.json
"""
import ctypes as C
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import quad_cases as Q  # noqa: E402

FN = C.CFUNCTYPE(C.c_double, C.c_double, C.c_void_p)


def main():
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libcaps_ref.so"))
    d, i = C.c_double, C.c_int
    lib.dqagi.restype = d
    lib.dqagi.argtypes = [FN, d, i, d, d, C.POINTER(d), C.POINTER(i), C.POINTER(i), C.c_void_p]
    lib.fcqs_semiinf.restype = d
    lib.fcqs_semiinf.argtypes = [FN, C.c_void_p, C.POINTER(d), C.POINTER(i), d, C.POINTER(i)]
    lib.psd.restype = i
    lib.psd.argtypes = [i, C.POINTER(d), C.POINTER(d)]
    out = dict(source="oracle/_ref/libcaps_ref.so (cquadpack dqagi, src/fcqs.c, src/psd.c)", qagi={}, fcqs={}, psd={})
    for name, (f, bound, inf) in Q.QAGI.items():
        cb = FN(lambda x, _u, f=f: f(x))
        for eps in Q.EPSRELS:
            ab, ne, ier = d(), i(), i()
            r = lib.dqagi(cb, bound, inf, 0.0, eps, C.byref(ab), C.byref(ne), C.byref(ier), None)
            out["qagi"]["%s_%g" % (name, eps)] = dict(result=r, abserr=ab.value, neval=ne.value, ier=ier.value)
    for name, (f, L) in Q.FCQS.items():
        cb = FN(lambda x, _u, f=f: f(x))
        eps, ne, ier = d(1e-10), i(), i()
        r = lib.fcqs_semiinf(cb, None, C.byref(eps), C.byref(ne), L, C.byref(ier))
        out["fcqs"][name] = dict(result=r, epsrel=eps.value, neval=ne.value, ier=ier.value)
    for N in list(range(1, 25)) + [40, 64]:
        xi, eta = (d * N)(), (d * N)()
        assert lib.psd(N, xi, eta) == 0
        out["psd"][str(N)] = dict(xi=list(xi), eta=list(eta))
    json.dump(out, open(os.path.join(HERE, "quad_golden.json"), "w"), indent=1)
    print({k: len(v) for k, v in out.items() if isinstance(v, dict)})


if __name__ == "__main__":
    main()
