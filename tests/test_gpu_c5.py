"""Randomised geometries: 64 draws from a fixed seed --
log-uniform R/L in [10, 500], T uniform in [0, 350] K, omega_p uniform in [7, 10] eV,
gamma uniform in [0.02, 0.05] eV, ldim = ceil(7 R/L) -- of which those with R/L <= 40 are
compared with the oracle at several (xi, m): FP64 to 1e-10, the mixed form to 5e-8."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HBAR, KB, CL = 1.0545718e-34, 1.38064852e-23, 299792458.0


def draws():
    rng = np.random.default_rng(0)
    out = []
    for _ in range(64):
        RbyL = math.exp(rng.uniform(math.log(10), math.log(500)))
        T = rng.uniform(0, 350)
        wp = rng.uniform(7, 10)
        ga = rng.uniform(0.02, 0.05)
        out.append((RbyL, T, wp, ga, int(math.ceil(7 * RbyL))))
    return out


CASES = [d for d in draws() if d[0] <= 40][:6]
_ORACLE = {}


@pytest.mark.parametrize("case", CASES, ids=["RbyL%.1f" % c[0] for c in CASES])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_random_geometry_vs_oracle(case, prec):
    import caps_gb300 as cg
    from oracle import binding as ob
    RbyL, T, wp, ga, ldim = case
    L = 1e-6
    R = RbyL * L
    Ts = 2 * math.pi * KB * (R + L) * max(T, 1.0) / (HBAR * CL)   # a Matsubara spacing (T -> 0: 1 K)
    xs = [Ts, 3.5 * Ts, 0.7]
    ms = [0, 3, 17]
    bx = [x for x in xs for _ in ms]
    bm = [m for _ in xs for m in ms]
    c = cg.Caps(R, L, ldim=ldim, detalg=cg.DETALG_LU)
    c.set_drude(wp, ga)
    c.set_precision(cg.PREC_MIXED if prec == "mixed" else cg.PREC_FP64)
    got, st = c.logdetD_batch(bx, bm)
    if case not in _ORACLE:
        _ORACLE[case] = ob.logdetD_batch(R, L, ldim, bx, bm, (wp, ga), threads=16)
    want = _ORACLE[case]
    tol = 1e-10 if prec == "fp64" else 5e-8
    for x, m, g, s, w in zip(bx, bm, got, st, want):
        assert s < 16, (case, x, m, s)
        assert abs(g - w) <= tol * max(1.0, abs(w)), (case, x, m, g, w)
