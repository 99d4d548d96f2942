"""Golden logdetD of the large-aspect workload from the unmodified reference library
(oracle/_ref/libcaps_ref.so): plasma model (omega_p = 9 eV, gamma = 0), R = 100 um,
L = 100 nm (R/L = 1000), ldim 6000 (matrices of dimension 12000), at three nodes of the
60-point Gauss-Laguerre rule in x = 2 xi L / c (xi (L+R)/c = x (L+R)/(2L)) and three m,
by the reference's LU and HODLR determinants.  Writes tests/golden/reference_c4.json.

    OPENBLAS_NUM_THREADS=1 python tests/golden/make_golden_c4.py     (~10 CPU-min per case)
"""
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden_energy import HBAR_EV, _init  # noqa: E402
import make_golden_energy as mge  # noqa: E402

R, L, LDIM, OMEGAP_EV = 1e-4, 1e-7, 6000, 9.0
NODES = (2, 9, 24)     # indices into the 60 Gauss-Laguerre abscissae
MS = (0, 60, 300)


def case(args):
    xi, m, detalg = args
    import ctypes as C
    lib = mge._lib
    c = lib.caps_init(R, L)
    lib.caps_set_ldim(c, LDIM)
    lib.caps_set_detalg(c, detalg)
    ud = (C.c_double * 2)(OMEGAP_EV / HBAR_EV, 0.0)
    lib.caps_set_epsilonm1(c, C.cast(lib.caps_epsilonm1_drude, C.c_void_p), C.cast(ud, C.c_void_p))
    t = time.time()
    v = lib.caps_logdetD(c, xi, m)
    lib.caps_free(c)
    return xi, m, detalg, v, time.time() - t


if __name__ == "__main__":
    x, w = np.polynomial.laguerre.laggauss(60)
    xis = [float(x[i]) * (L + R) / (2 * L) for i in NODES]
    jobs = [(xi, m, alg) for xi in xis for m in MS for alg in (1, 0)]
    with mp.Pool(int(os.environ.get("PROCS", "8")), initializer=_init) as pool:
        res = pool.map(case, jobs, chunksize=1)
    cases = []
    for xi in xis:
        for m in MS:
            row = dict(R=R, L=L, ldim=LDIM, omegap_eV=OMEGAP_EV, gamma_eV=0.0, xi=xi, m=m)
            for (x_, m_, alg, v, dt) in res:
                if x_ == xi and m_ == m:
                    row["LU" if alg == 1 else "HODLR"] = v
                    row[("LU" if alg == 1 else "HODLR") + "_seconds"] = dt
            cases.append(row)
            print(row, file=sys.stderr)
    json.dump(dict(source="oracle/_ref/libcaps_ref.so via tests/golden/make_golden_c4.py",
                   gauss_laguerre_nodes=[int(i) for i in NODES], cases=cases),
              open(os.path.join(HERE, "reference_c4.json"), "w"), indent=1)
