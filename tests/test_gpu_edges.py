"""Edge cases of the batch interface: an empty batch, batches whose results must not depend
on their composition (order, duplicates, ragged mixes of frequencies and m against single
calls -- bitwise, as every matrix is computed from its own (xi, m) alone), and the
reference's contract violations, which abort as its TERMINATE does (src/include/utils.h:31:
xi <= 0, src/libcaps.c:952) or as this library's own limit does (an l window beyond 27000),
checked before any kernel runs; those run in child processes."""
import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cg():
    import caps_gb300
    return caps_gb300


def test_empty_batch(cg):
    c = cg.Caps(20e-6, 1e-6, ldim=40)
    out = (C.c_double * 1)(7.0)
    assert cg.lib.caps_logdetD_batch(c._h, None, None, 0, out, None) == 0
    assert out[0] == 7.0


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_order_and_duplicates(cg, prec):
    rng = np.random.default_rng(5)
    xi = list(rng.uniform(0.5, 40.0, 24))
    ms = [int(x) for x in rng.integers(0, 30, 24)]
    xi += xi[:4]          # duplicates
    ms += ms[:4]
    c = cg.Caps(20e-6, 1e-6, ldim=140)
    c.set_drude(9.0, 0.035)
    c.set_precision(prec)
    a, sa = c.logdetD_batch(xi, ms)
    perm = rng.permutation(len(xi))
    b, sb = c.logdetD_batch([xi[i] for i in perm], [ms[i] for i in perm])
    assert max(sa) < 16 and max(sb) < 16
    assert np.array_equal(a[perm], b)
    assert np.array_equal(a[:4], a[-4:])


def test_ragged_batch_equals_single_calls(cg):
    """one batch mixing frequencies and m up to the shifted l windows of R/L=150 (m > 68)
    against one call of caps_logdetD per matrix"""
    c = cg.Caps(150e-6, 1e-6, ldim=200)
    c.set_drude(9.0, 0.035)
    xi = [124.3, 124.3, 248.6, 1118.7, 372.9, 124.3]
    ms = [0, 150, 69, 3, 120, 68]
    out, st = c.logdetD_batch(xi, ms)
    for x, m, v in zip(xi, ms, out):
        assert c.logdetD(x, m) == v, (x, m)


def _child(code):
    return subprocess.run([sys.executable, "-c", "import sys; sys.path.insert(0, %r)\n" % ROOT + code], capture_output=True,
                          text=True, timeout=300)


def test_nonpositive_frequency_aborts():
    r = _child("import caps_gb300 as cg\nc = cg.Caps(20e-6, 1e-6, ldim=40)\nc.logdetD(0.0, 0)\nprint('returned')")
    assert r.returncode != 0 and "returned" not in r.stdout
    assert "Matsubara frequency must be positive" in r.stderr


def test_window_beyond_limit_aborts():
    r = _child("import caps_gb300 as cg\nc = cg.Caps(20e-6, 1e-6, ldim=26000)\nc.logdetD(1.0, 2000)\nprint('returned')")
    assert r.returncode != 0 and "returned" not in r.stdout
    assert "l window beyond 27000" in r.stderr
