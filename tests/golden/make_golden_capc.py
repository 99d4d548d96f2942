"""Golden cylinder-plane values from the unmodified reference (oracle/_ref): the
reference's own capc program (src/capc.cpp) compiled behind the C wrapper
oracle/capc_ref.cpp -- CasimirCP::logdet and CasimirCP::energy -- and the integer-order
Bessel functions of the reference library (src/bessel.c).

    make -f oracle/Makefile.ref REF=<reference tree> -j8
    python tests/golden/make_golden_capc.py      # writes tests/golden/capc_golden.json
"""
import ctypes as C
import json
import math
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(ROOT, "oracle", "_ref")
HODLR, LU = 0, 1  # detalg_t

# (R, d, lmax): R/d = 10 and 50 at the capc CLI's eta = 6, and the constructor's
# minimum dimension 25 at R/d = 1
GEOMS = [(1.0, 0.1, 60), (1.0, 0.02, 300), (1.0, 1.0, 25)]
QS = {0: [1e-4, 1e-3, 0.05, 0.5, 1.0, 3.0, 5.0, 10.0, 30.0, 100.0, 400.0],
      1: [0.01, 0.5, 2.0, 5.0, 25.0, 100.0],
      2: [1e-3, 0.1, 0.7, 2.0, 8.0]}
ENERGY = [(0, "D"), (0, "N"), (1, "D"), (1, "N")]
EPSREL = 1e-8  # capc default
XS = [1e-9, 1e-5, 1e-3, 0.1, 0.5, 1, 2, 3, 5, 7.9, 8, 10, 30, 100, 500, 799, 800, 1500, 2500, 1e4, 1e5]
NS = [2, 3, 5, 10, 30, 60, 99, 100, 101, 150, 300, 1000, 2401]


def main():
    lib = C.CDLL(os.path.join(REF, "libcaps_ref.so"))
    capc = C.CDLL(os.path.join(REF, "libcapc_ref.so"))
    d, i = C.c_double, C.c_int
    for f in ("bessel_logI0", "bessel_logI1", "bessel_logK0", "bessel_logK1"):
        getattr(lib, f).restype, getattr(lib, f).argtypes = d, [d]
    for f in ("bessel_logIn", "bessel_logKn"):
        getattr(lib, f).restype, getattr(lib, f).argtypes = d, [i, d]
    capc.capc_ref_logdet.restype, capc.capc_ref_logdet.argtypes = d, [d, d, i, d, C.c_char, i]
    capc.capc_ref_energy.restype, capc.capc_ref_energy.argtypes = d, [d, d, i, C.c_char, d, i]

    out = {"bessel01": [], "besseln": [], "logdet": [], "energy": []}
    for x in XS:
        out["bessel01"].append({"x": x, **{f: getattr(lib, "bessel_" + f)(x)
                                         for f in ("logI0", "logI1", "logK0", "logK1")}})
    for n in NS:
        for x in XS:
            out["besseln"].append({"n": n, "x": x, "logIn": lib.bessel_logIn(n, x), "logKn": lib.bessel_logKn(n, x)})
    for g, (R, dd, lmax) in enumerate(GEOMS):
        for q in QS[g]:
            for dn in "DN":
                row = {"R": R, "d": dd, "lmax": lmax, "q": q, "DN": dn,
                       "hodlr": capc.capc_ref_logdet(R, dd, lmax, q, dn.encode(), HODLR)}
                if g != 1:
                    row["lu"] = capc.capc_ref_logdet(R, dd, lmax, q, dn.encode(), LU)
                out["logdet"].append(row)
    for g, p in ENERGY:
        R, dd, lmax = GEOMS[g]
        t = time.time()
        E = capc.capc_ref_energy(R, dd, lmax, p.encode(), EPSREL, HODLR)
        out["energy"].append({"R": R, "d": dd, "lmax": lmax, "p": p, "epsrel": EPSREL, "E": E,
                              "E_over_pfa_dn": E / (-math.pi ** 3 / 1920 * math.sqrt(R / (2 * dd)) / dd ** 2),
                              "ref_seconds": round(time.time() - t, 3)})
        print(out["energy"][-1], flush=True)
    with open(os.path.join(HERE, "capc_golden.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
