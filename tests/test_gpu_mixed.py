"""Mixed-precision factorisation (CAPS_PREC_MIXED): delta-form FP32 Cholesky with
FP64 pivot logarithms and an FP64 trace correction.  Bars: per matrix
|dlogdetD| <= 5e-8 max(1,|logdetD|) against the reference's values, and the
free energy within |dE/E| <= 1e-6 of the FP64 oracle."""
import pytest

from conftest import rel, relx

pytestmark = pytest.mark.gpu
TOL_MIXED = 5e-8


@pytest.fixture(scope="module")
def cg():
    import caps_gb300
    return caps_gb300


def test_mixed_unit_vectors_RbyL100(cg, unit_vectors):
    cases = [v for v in unit_vectors["test_logdetD"]["cases"] if v["ldim"] == 500]
    c = cg.Caps(1.0, 0.01, ldim=500)
    c.set_precision(cg.PREC_MIXED)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    for v, got, s in zip(cases, out, st):
        assert s < 16, (v, s)
        assert abs(got - v["logdetD"]) <= TOL_MIXED * max(1.0, abs(v["logdetD"])), (v, got)


def test_mixed_unit_vectors_RbyL1000(cg, unit_vectors):
    """test_logdetD.c:77-102 in the mixed form: R/L=1000, ldim=10000 (matrices of dimension
    20000, degrees up to ~21000 in the float-float K recurrence)"""
    cases = [v for v in unit_vectors["test_logdetD"]["cases"] if v["ldim"] == 10000]
    c = cg.Caps(1.0, 0.001, ldim=10000)
    c.set_precision(cg.PREC_MIXED)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    for v, got, s in zip(cases, out, st):
        assert s < 16, (v, s)
        assert abs(got - v["logdetD"]) <= TOL_MIXED * max(1.0, abs(v["logdetD"])), (v, got)


@pytest.mark.parametrize("name", ["drude_RbyL150_ldim1050", "pr_RbyL50_ldim350", "drude_RbyL20_ldim140"])
def test_mixed_vs_reference_fixtures(cg, ref_values, name):
    if name not in ref_values:
        pytest.skip("fixture set not generated")
    cases = ref_values[name]
    c0 = cases[0]
    c = cg.Caps(c0["R"], c0["L"], ldim=c0["ldim"], detalg=cg.DETALG_LU)
    if c0["drude"]:
        c.set_drude(*c0["drude"])
    c.set_precision(cg.PREC_MIXED)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    for v, got, s in zip(cases, out, st):
        assert s < 16
        assert abs(got - v["LU"]) <= TOL_MIXED * max(1.0, abs(v["LU"])), (v, got)


def test_mixed_free_energy(cg):
    from oracle import binding as ob
    R, L, T, ldim = 10e-6, 1e-6, 300.0, 70
    for drude in (None, (9.0, 0.035)):
        c = cg.Caps(R, L, ldim=ldim, detalg=cg.DETALG_LU)
        if drude:
            c.set_drude(*drude)
        c.set_precision(cg.PREC_MIXED)
        E, info = c.free_energy(T)
        Eo, _ = ob.free_energy(R, L, ldim, T, drude, threads=8)
        assert abs(E - Eo) <= 1e-6 * abs(Eo), (E, Eo)


def test_mixed_dense_M_reference(cg, ref_values):
    """the float-float q-sums of the mixed form keep element-level parity"""
    import numpy as np
    for v in ref_values["dense_M"]:
        c = cg.Caps(v["R"], v["L"], ldim=v["ldim"])
        if v["drude"]:
            c.set_drude(*v["drude"])
        c.set_precision(cg.PREC_MIXED)
        M = c.M(v["xi"], v["m"])
        Mr = np.array(v["M"])
        assert np.abs(M - Mr).max() < 1e-10 * np.abs(Mr).max(), v["m"]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("drude", [None, (9.0, 0.035)])
def test_batch_order_and_grouping_independent(cg, prec, drude):
    """The library runs a batch in (m, xi) order and, in the mixed form, pairs
    consecutive frequencies of one m on a shared a_q recurrence.  Each result must be
    independent of the caller's order and of its partner: bitwise equal to the same
    matrix computed alone."""
    import numpy as np
    c = cg.Caps(20e-6, 1e-6, ldim=140)
    if drude:
        c.set_drude(*drude)
    c.set_precision(cg.PREC_MIXED if prec == "mixed" else cg.PREC_FP64)
    xis = [0.7, 3.1, 9.4, 21.0, 3.1, 0.7]
    ms = [0, 5, 5, 5, 12, 12]
    rng = np.random.default_rng(3)
    perm = rng.permutation(len(xis))
    out, st = c.logdetD_batch([xis[i] for i in perm], [ms[i] for i in perm])
    assert all(s < 16 for s in st)
    for k, i in enumerate(perm):
        alone = c.logdetD(xis[i], ms[i])
        assert out[k] == alone, (xis[i], ms[i], out[k], alone)


def test_mixed_trace_rule_first(cg):
    """The mixed form applies the trace rule (matrix.c:62-82) to the diagonal before it
    assembles anything else, and assembles in full only the matrices that the rule leaves
    undecided.  The decision and the values must be those of the FP64 form, which
    assembles every matrix; each result must also be bitwise the one of the matrix
    computed alone (the full q-sums then group a different set of frequencies)."""
    import numpy as np
    xis = [1.0, 30.0, 150.0, 400.0]
    ms = [0, 3, 60, 130]
    X = [x for x in xis for _ in ms]
    M = [m for _ in xis for m in ms]
    c = cg.Caps(20e-6, 1e-6, ldim=140)
    c.set_drude(9.0, 0.035)
    ref, st_ref = c.logdetD_batch(X, M)
    c.set_precision(cg.PREC_MIXED)
    out, st = c.logdetD_batch(X, M)
    assert list(st) == list(st_ref)
    assert 1 in set(st) and 3 in set(st), st   # both trace-rule and factored matrices
    for x, m, a, b, s in zip(X, M, out, ref, st):
        if s == 1:  # -tr M: float-float elements, relative error far below the FP32 bar
            assert abs(a - b) <= 1e-6 * abs(b), (x, m, a, b)
        else:
            assert abs(a - b) <= TOL_MIXED * max(1.0, abs(b)), (x, m, a, b)
    for k in np.random.default_rng(5).permutation(len(X))[:6]:
        assert out[k] == c.logdetD(X[k], M[k]), (X[k], M[k])


@pytest.mark.parametrize("variant", ["", "CAPS_MIXED_REGSTAGE", "CAPS_MIXED_NOPIPE", "CAPS_MIXED_MMASYNC", "CAPS_MIXED_SIMT"])
def test_mixed_update_variants(variant):
    """Every trailing-update variant of the mixed factorisation (image-fed persistent
    kernels by default; register staging, one CTA per tile, the single-level mma.sync and
    FFMA forms behind environment switches, read once per process) against the FP64 form,
    on matrices of dimension 700 (two 256-column panels and a partial third)."""
    import json
    import os
    import subprocess
    import sys
    code = (
        "import json, caps_gb300 as cg\n"
        "c = cg.Caps(50e-6, 1e-6, ldim=350)\n"
        "c.set_drude(9.0, 0.035)\n"
        "x = [0.8, 3.0, 3.0, 12.0]; m = [0, 0, 7, 2]\n"
        "ref, _ = c.logdetD_batch(x, m)\n"
        "c.set_precision(cg.PREC_MIXED)\n"
        "out, st = c.logdetD_batch(x, m)\n"
        "print(json.dumps({'ref': list(ref), 'out': list(out), 'st': [int(s) for s in st]}))\n")
    env = dict(os.environ)
    for k in ["CAPS_MIXED_REGSTAGE", "CAPS_MIXED_NOPIPE", "CAPS_MIXED_MMASYNC", "CAPS_MIXED_SIMT"]:
        env.pop(k, None)
    if variant:
        env[variant] = "1"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env["PYTHONPATH"] = root + os.pathsep + env.get("PYTHONPATH", "")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert all(s == 3 for s in d["st"]), d["st"]  # all factored
    for a, b in zip(d["out"], d["ref"]):
        assert abs(a - b) <= TOL_MIXED * max(1.0, abs(b)), (variant, a, b)


def test_mixed_correction_error_by_dimension(cg, unit_vectors):
    """the per-matrix error of the mixed form's first-order correction (log det A ~
    2 sum log1p(Lam_jj) + tr Delta) against the FP64 form as the dimension grows: the
    hardest matrices (lowest frequency, m = 0 ..) at dimension 2100 (Drude gold, R/L=150),
    12000 (plasma, R/L=1000, L=100 nm) and 20000 (perfect reflectors, R/L=1000, the
    reference's own unit-test geometry); each within 5e-8 max(1, |logdetD|)"""
    cases = {
        2100: (150e-6, 1e-6, 1050, (9.0, 0.035), [124.298] * 4, [0, 5, 20, 60]),
        12000: (1e-4, 1e-7, 6000, (9.0, 0.0), [50.05, 500.5, 2502.5, 500.5], [0, 0, 0, 60]),
        20000: (1.0, 0.001, 10000, None, [1.0, 1.0, 10.0], [0, 40, 0]),
    }
    worst = {}
    for dim, (R, L, ldim, drude, xi, ms) in cases.items():
        out = {}
        for prec in (cg.PREC_FP64, cg.PREC_MIXED):
            c = cg.Caps(R, L, ldim=ldim, detalg=cg.DETALG_LU)
            if drude:
                c.set_drude(*drude)
            c.set_precision(prec)
            v, st = c.logdetD_batch(xi, ms)
            assert max(st) < 16, (dim, prec, list(st))
            out[prec] = v
        err = [abs(a - b) / max(1.0, abs(b)) for a, b in zip(out[cg.PREC_MIXED], out[cg.PREC_FP64])]
        worst[dim] = max(err)
        print("dimension %d: logdetD %s, mixed-form error %s" % (dim, ["%.6g" % x for x in out[cg.PREC_FP64]],
                                                                  ["%.1e" % e for e in err]))
    assert all(e <= TOL_MIXED for e in worst.values()), worst
