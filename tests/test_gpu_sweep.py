"""The mixed form's matrix assembly by the I recurrence (sweep.cu: q-sums of 4L seed pairs,
the rest of the table by the three-term Legendre recurrence in both degrees, elements formed
as the rows appear) on inputs the workload tests do not reach: the plasma model at low and
high frequencies, perfect reflectors at m = 0, the smallest windows, and the two sides of the
largest window whose rows fit the kernel's shared-memory ring (beyond it the full q-sum table
is used).  Each is compared with the FP64 form (q-sums of every pair, scaled doubles) at the
mixed form's per-matrix bar, |d logdetD| <= 5e-8 max(1, |logdetD|)."""
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu
TOL = 5e-8


@pytest.fixture(scope="module")
def cg():
    import caps_gb300
    return caps_gb300


ST_FACTOR = 3  # status of a matrix assembled in full and factorised (not ended by the trace rule)


def both(cg, R, L, ldim, xi, ms, material=None, min_factored=1):
    out = {}
    for prec in (cg.PREC_FP64, cg.PREC_MIXED):
        c = cg.Caps(R, L, ldim=ldim, detalg=cg.DETALG_LU)
        if material:
            c.set_drude(*material)
        c.set_precision(prec)
        v, st = c.logdetD_batch(xi, ms)
        assert max(st) < 16, (prec, list(st))
        # the cases must reach the assembly (the recurrence), not only the trace rule
        assert sum(int(s) == ST_FACTOR for s in st) >= min_factored, (prec, list(st))
        out[prec] = v
    return out[cg.PREC_FP64], out[cg.PREC_MIXED]


def test_sweep_plasma_low_and_high_frequency(cg):
    """plasma (wp = 9 eV, gamma = 0), R/L = 100, L = 100 nm, ldim 700 (dimension 1400)"""
    xi = [0.05, 0.05, 0.05, 2.0, 2.0, 40.0, 40.0, 400.0, 400.0]
    ms = [0, 1, 12, 0, 25, 3, 60, 1, 150]
    a, b = both(cg, 1e-5, 1e-7, 700, xi, ms, (9.0, 0.0), min_factored=5)
    for x, m, u, v in zip(xi, ms, a, b):
        assert rel(v, u) <= TOL, (x, m, u, v)


def test_sweep_perfect_reflector_m0(cg):
    """perfect reflectors (I_TE = -I_TM), R/L = 20, every m up to 8 at three frequencies"""
    xi = [x for x in (0.3, 3.0, 30.0) for m in range(9)]
    ms = [m for x in (0.3, 3.0, 30.0) for m in range(9)]
    a, b = both(cg, 20e-6, 1e-6, 140, xi, ms, min_factored=12)
    for x, m, u, v in zip(xi, ms, a, b):
        assert rel(v, u) <= TOL, (x, m, u, v)


@pytest.mark.parametrize("ldim", [4, 9])
def test_sweep_smallest_windows(cg, ldim):
    """windows of a few l (the ring's first rows, the first column, the zero row of m = 0)"""
    xi = [0.5, 0.5, 0.5, 5.0]
    ms = [0, 1, 3, 2]
    a, b = both(cg, 5e-6, 1e-6, ldim, xi, ms, (9.0, 0.035))
    for x, m, u, v in zip(xi, ms, a, b):
        assert rel(v, u) <= TOL, (x, m, u, v)


@pytest.mark.parametrize("ldim", [2200, 2400])
def test_sweep_ring_limit(cg, ldim):
    """ldim 2200 (the recurrence sweep: 104 bytes of shared memory per l) and 2400 (beyond the
    ring: the full q-sum table), Drude, R/L = 400, dimensions 4400 and 4800"""
    xi = [2.0, 2.0, 20.0]
    ms = [0, 4, 1]
    a, b = both(cg, 400e-6, 1e-6, ldim, xi, ms, (9.0, 0.035), min_factored=2)
    for x, m, u, v in zip(xi, ms, a, b):
        assert rel(v, u) <= TOL, (x, m, u, v)
