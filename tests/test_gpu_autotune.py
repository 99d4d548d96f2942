"""The autotuner (caps_gpu_autotune): it times the candidate schedules on a probe batch of the
caller's workload and keeps the fastest.  Whatever it picks, results stay within the form's
bar against the reference library's values: the mixed form's trailing-update schedules differ
only in the rounding of the FP32 update, the FP64 paths (dense, HODLR) only by HODLR's
compression tolerance."""
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(0, 1e-10), (1, 5e-8)])
def test_autotune_keeps_results(ref_values, prec, tol):
    import caps_gb300 as cg
    cases = ref_values["pr_RbyL50_ldim350"]
    v0 = cases[0]
    c = cg.Caps(v0["R"], v0["L"], ldim=v0["ldim"])      # DETALG_HODLR
    c.set_precision(prec)
    chosen, times = c.autotune(v0["xi"], nprobe=6)
    assert len(times) == (4 if prec == cg.PREC_MIXED else 2) and 0 <= chosen < len(times)
    assert all(t > 0 for t in times) and times[chosen] == min(times)
    out, st = c.logdetD_batch([v["xi"] for v in cases], [v["m"] for v in cases])
    for v, got, s in zip(cases, out, st):
        assert s < 16
        assert rel(got, v["HODLR"]) < tol, (prec, chosen, v["xi"], v["m"], got, v["HODLR"])
