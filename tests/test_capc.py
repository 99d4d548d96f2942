"""Cylinder-plane geometry (the reference's capc program, src/capc.cpp) and the
integer-order Bessel functions it uses (src/bessel.c:283-633).

Golden values come from the reference itself (tests/golden/make_golden_capc.py runs
its CasimirCP class and its bessel_* functions).  CPU tests pin the oracle and the
library's host-side Bessel functions against them; the GPU tests check the library's
batched logdet and T = 0 energy against the golden values and the oracle.
Tolerances: Bessel logs 1e-13 max(1, |v|); logdet 1e-10 max(1, |v|), the reference's
own test bar (test_logdetD.c:57); energies 1e-10 relative."""
import json
import math
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
BTOL, TOL = 1e-13, 1e-10


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "capc_golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def ob():
    from oracle import binding
    return binding


@pytest.fixture(scope="module")
def cg():
    import caps_gb300
    return caps_gb300


def err(a, b):
    if math.isinf(b) and a == b:
        return 0.0
    return abs(a - b) / max(1.0, abs(b))


def _bessel_cases(golden):
    for r in golden["bessel01"]:
        for f in ("logI0", "logI1", "logK0", "logK1"):
            yield ("bessel_" + f, (r["x"],), r[f])
    for r in golden["besseln"]:
        yield ("bessel_logIn", (r["n"], r["x"]), r["logIn"])
        yield ("bessel_logKn", (r["n"], r["x"]), r["logKn"])


def test_oracle_bessel_golden(golden, ob):
    bad = [(f, a, v, getattr(ob.lib, "oracle_" + f)(*a)) for f, a, v in _bessel_cases(golden)
           if err(getattr(ob.lib, "oracle_" + f)(*a), v) > BTOL]
    assert not bad, bad[:5]


def test_library_bessel_golden(golden, cg):
    """host functions of the C-ABI library; no GPU involved"""
    bad = [(f, a, v, getattr(cg.lib, f)(*a)) for f, a, v in _bessel_cases(golden) if err(getattr(cg.lib, f)(*a), v) > BTOL]
    assert not bad, bad[:5]


def test_library_bessel_edges(cg):
    L = cg.lib
    assert L.bessel_logI0(0.0) == 0.0
    assert L.bessel_logIn(3, 0.0) == -math.inf
    assert math.isnan(L.bessel_logI1(0.0)) and math.isnan(L.bessel_logK0(0.0)) and math.isnan(L.bessel_logKn(4, -1.0))
    assert L.bessel_logIn(-7, 3.0) == L.bessel_logIn(7, 3.0) and L.bessel_logKn(-7, 3.0) == L.bessel_logKn(7, 3.0)
    # recurrences: K_{n+1} = K_{n-1} + 2n/x K_n, I_{n-1} = I_{n+1} + 2n/x I_n
    x, n = 3.7, 12
    k = [math.exp(L.bessel_logKn(j, x)) for j in (n - 1, n, n + 1)]
    i = [math.exp(L.bessel_logIn(j, x)) for j in (n - 1, n, n + 1)]
    assert abs(k[2] - k[0] - 2 * n / x * k[1]) < 1e-14 * k[2]
    assert abs(i[0] - i[2] - 2 * n / x * i[1]) < 1e-14 * i[0]


def test_lmax_and_pfa(cg):
    assert cg.capc_lmax(1.0, 0.1) == 60 and cg.capc_lmax(1.0, 1.0) == 25 and cg.capc_lmax(1.0, 0.02, 5.0) == 250
    assert abs(cg.lib.caps_capc_pfa(1.0, 0.1) - (-math.pi ** 3 / 1920 * math.sqrt(5.0) / 0.01)) < 1e-15


def test_oracle_capc_golden(golden, ob):
    for r in golden["logdet"]:
        for key, hodlr in (("hodlr", 1), ("lu", 0)):
            if key not in r:
                continue
            v = ob.lib.oracle_capc_logdet(r["R"], r["d"], r["lmax"], r["q"], r["DN"].encode(), hodlr)
            assert err(v, r[key]) < TOL, (r, key, v)


@pytest.mark.gpu
def test_gpu_capc_logdet_golden(golden, cg):
    groups = {}
    for r in golden["logdet"]:
        groups.setdefault((r["R"], r["d"], r["lmax"], r["DN"]), []).append(r)
    for (R, d, lmax, DN), rows in groups.items():
        q = np.array([r["q"] for r in rows])
        for key in ("hodlr", "lu"):
            if key not in rows[0]:
                continue
            got = cg.capc_logdet(R, d, q, DN, lmax, key.upper())
            for r, v in zip(rows, got):
                assert err(v, r[key]) < TOL, (r, key, v)


@pytest.mark.gpu
def test_gpu_capc_logdet_oracle_random(cg, ob):
    rng = np.random.default_rng(7)
    for R, d in ((1.0, 0.1), (2.0, 0.05)):
        lmax = cg.capc_lmax(R, d)
        q = np.exp(rng.uniform(np.log(1e-3), np.log(300.0), 12))
        for DN in "DN":
            got = cg.capc_logdet(R, d, q, DN, lmax)
            for qq, v in zip(q, got):
                o = ob.lib.oracle_capc_logdet(R, d, lmax, float(qq), DN.encode(), 1)
                assert err(v, o) < TOL, (R, d, DN, qq, v, o)


@pytest.mark.gpu
def test_gpu_capc_batch_matches_single(cg):
    q = np.array([0.02, 0.3, 1.0, 4.0, 11.0, 50.0])
    batch = cg.capc_logdet(1.0, 0.1, q, "N", 60)
    single = [cg.capc_logdet(1.0, 0.1, float(x), "N", 60) for x in q]
    assert np.array_equal(batch, np.array(single))
    # 'd' is Dirichlet, any other letter Neumann (capc.cpp:51-53)
    assert cg.capc_logdet(1.0, 0.1, 1.0, "d", 60) == cg.capc_logdet(1.0, 0.1, 1.0, "D", 60)
    assert cg.capc_logdet(1.0, 0.1, 1.0, "x", 60) == cg.capc_logdet(1.0, 0.1, 1.0, "N", 60)
    assert cg.lib.caps_capc_logdet_batch(1.0, 0.1, 60, None, 0, b"D", 0, None) == 0


@pytest.mark.gpu
def test_gpu_capc_logdet_limits(cg):
    # large q: every element underflows, the trace shortcut gives -tr -> 0
    assert cg.capc_logdet(1.0, 0.1, 1e4, "D", 60) == 0.0
    # the logdet is negative and grows in magnitude towards small q
    v = cg.capc_logdet(1.0, 0.1, np.array([10.0, 1.0, 0.1, 0.01]), "D", 60)
    assert np.all(v < 0) and np.all(np.diff(v) < 0)


@pytest.mark.gpu
def test_gpu_capc_energy_golden(golden, cg):
    for r in golden["energy"]:
        E, neval, ier = cg.capc_energy_T0(r["R"], r["d"], r["p"], r["lmax"], r["epsrel"])
        assert ier == 0 and neval > 0
        assert abs(E - r["E"]) < TOL * abs(r["E"]), (r, E)
