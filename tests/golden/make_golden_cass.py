"""Golden sphere-sphere values from the unmodified reference library (oracle/_ref): the
steps of the reference's cass program (src/cass.c:23-92, 183-219) restated around the
library's own functions -- caps_M_init/caps_M_elem for M in cass's block layout,
matrix_mult for M^2, matrix_trace, matrix_logdet_dense(M^2, -1, DETALG_LU), and dqagi for
the T = 0 integral -- with the m loop of each frequency farmed out in chunks (summed in m
order, so the pool size does not change the result).

    python tests/golden/make_golden_cass.py      # writes tests/golden/cass_golden.json
"""
import ctypes as C
import json
import math
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref", "libcaps_ref.so")
R, D = 10e-6, 1e-6           # sphere radius, separation
L = D / 2
LDIM = int(max(20, R / D * 5))  # cass default (eta = 5)
CUTOFF, EPSREL = 1e-10, 1e-6    # cass defaults
_lib = None


class Matrix(C.Structure):
    _fields_ = [("dim", C.c_size_t), ("dim2", C.c_size_t), ("lda", C.c_size_t), ("M", C.POINTER(C.c_double))]


def _init():
    global _lib
    os.environ["OPENBLAS_NUM_THREADS"] = "1"
    _lib = C.CDLL(REF)
    vp, d, i = C.c_void_p, C.c_double, C.c_int
    _lib.caps_init.restype = vp
    _lib.caps_init.argtypes = [d, d]
    _lib.caps_set_ldim.argtypes = [vp, i]
    _lib.caps_set_detalg.argtypes = [vp, i]
    _lib.caps_set_epsrel.argtypes = [vp, d]
    _lib.caps_free.argtypes = [vp]
    _lib.caps_estimate_lminmax.argtypes = [vp, i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
    _lib.caps_M_init.restype = vp
    _lib.caps_M_init.argtypes = [vp, i, d]
    _lib.caps_M_elem.restype = d
    _lib.caps_M_elem.argtypes = [vp, i, i, C.c_char, C.c_char]
    _lib.caps_M_free.argtypes = [vp]
    _lib.matrix_alloc.restype = C.POINTER(Matrix)
    _lib.matrix_alloc.argtypes = [C.c_size_t]
    _lib.matrix_free.argtypes = [C.POINTER(Matrix)]
    _lib.matrix_mult.restype = C.POINTER(Matrix)
    _lib.matrix_mult.argtypes = [C.POINTER(Matrix), C.POINTER(Matrix), d]
    _lib.matrix_trace.restype = d
    _lib.matrix_trace.argtypes = [C.POINTER(Matrix)]
    _lib.matrix_logdet_dense.restype = d
    _lib.matrix_logdet_dense.argtypes = [C.POINTER(Matrix), d, i]


def logdetD2(args):
    """cass.c:23-64"""
    m, xi_ = args
    c = _lib.caps_init(R, L)
    _lib.caps_set_epsrel(c, 1e-9)   # cass sets its iepsrel default
    _lib.caps_set_ldim(c, LDIM)
    _lib.caps_set_detalg(c, 1)      # DETALG_LU
    lmin, lmax = C.c_size_t(), C.c_size_t()
    _lib.caps_estimate_lminmax(c, m, C.byref(lmin), C.byref(lmax))
    ldim = lmax.value - lmin.value
    M = _lib.matrix_alloc(2 * ldim)
    lda = M.contents.lda
    a = M.contents.M
    obj = _lib.caps_M_init(c, m, xi_)
    for i in range(ldim):
        l1 = i + lmin.value
        for j in range(ldim):
            l2 = j + lmin.value
            a[i * lda + j] = _lib.caps_M_elem(obj, l1, l2, b"E", b"E")
            a[i * lda + j + ldim] = _lib.caps_M_elem(obj, l1, l2, b"E", b"M")
            a[(i + ldim) * lda + j] = _lib.caps_M_elem(obj, l1, l2, b"M", b"E")
            a[(i + ldim) * lda + j + ldim] = _lib.caps_M_elem(obj, l1, l2, b"M", b"M")
    _lib.caps_M_free(obj)
    M2 = _lib.matrix_mult(M, M, 1.0)
    _lib.matrix_free(M)
    trace2 = _lib.matrix_trace(M2)
    if trace2 < 1e-8:
        r = -trace2
    else:
        r = _lib.matrix_logdet_dense(M2, -1.0, 1)
    _lib.matrix_free(M2)
    _lib.caps_free(c)
    return r


def kahan(v):
    s = c = 0.0
    for x in v:
        y = x - c
        t = s + y
        c = (t - s) - y
        s = t
    return s


def main():
    procs = int(os.environ.get("PROCS", "8"))
    _init()
    d, i = C.c_double, C.c_int
    FN = C.CFUNCTYPE(d, d, C.c_void_p)
    _lib.dqagi.restype = d
    _lib.dqagi.argtypes = [FN, d, i, d, d, C.POINTER(d), C.POINTER(i), C.POINTER(i), C.c_void_p]
    samples = [(m, x) for x in (0.3, 2.0, 9.0, 40.0) for m in (0, 1, 4)]
    evals = []
    with mp.Pool(procs, initializer=_init) as pool:
        values = pool.map(logdetD2, samples)

        def integrand(y, _u):
            """cass.c:66-92"""
            xi_ = y * (L + R) / (2 * L)
            terms, m0 = [], 0
            while True:
                vals = pool.map(logdetD2, [(m, xi_) for m in range(m0, m0 + procs)])
                stop = False
                for v in vals:
                    terms.append(v)
                    if v == 0 or v / terms[0] < CUTOFF:
                        stop = True
                        break
                if stop:
                    break
                m0 += procs
            t = terms + [0.0] * (4096 - len(terms))
            r = 2 * kahan(t) - terms[0]
            evals.append((xi_, r))
            return r
        cb = FN(integrand)
        ab, ne, ier = d(), i(), i()
        integral = _lib.dqagi(cb, 0.0, 1, 0.0, EPSREL, C.byref(ab), C.byref(ne), C.byref(ier), None)
    out = dict(source="oracle/_ref/libcaps_ref.so via tests/golden/make_golden_cass.py (steps of src/cass.c)",
               R=R, d=D, ldim=LDIM, cutoff=CUTOFF, epsrel=EPSREL,
               samples=[dict(m=m, xi=x, logdetD2=v) for (m, x), v in zip(samples, values)],
               E=integral / (2 * math.pi), neval=ne.value, ier=ier.value, abserr=ab.value,
               xi=[e[0] for e in evals], F=[e[1] for e in evals])
    json.dump(out, open(os.path.join(HERE, "cass_golden.json"), "w"), indent=1)
    print(out["E"], out["neval"], out["ier"], file=sys.stderr)


if __name__ == "__main__":
    main()
