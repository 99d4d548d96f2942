"""The drop-in from C: tests/c_caller/drop_in.c is written against include/libcaps.h the
way the reference's own callers use the API (src/caps_logdetD.c:176-215,
examples/AuAl.c) and linked against libcaps_gb300.so with a plain C99 compiler.  Building
it checks the header, the struct layout it relies on and the link line; running it (on a
GPU) checks its results against the reference's values."""
import os
import subprocess

import pytest

from conftest import ROOT, relx

SRC = os.path.join(ROOT, "tests", "c_caller", "drop_in.c")


def build(tmp_path):
    import caps_gb300
    libdir = os.path.dirname(caps_gb300.LIB_PATH)
    exe = str(tmp_path / "drop_in")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I" + os.path.join(ROOT, "include"), SRC,
           caps_gb300.LIB_PATH, "-Wl,-rpath," + libdir, "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_caller_builds(tmp_path):
    assert os.path.exists(build(tmp_path))


@pytest.mark.gpu
def test_c_caller_matches_reference(tmp_path, ref_values, unit_vectors):
    exe = build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = {k: float(v) for k, v in (ln.split() for ln in r.stdout.splitlines())}
    assert out["init_invalid_is_null"] == 1 and out["set_ldim_zero"] == 0 and out["set_ldim"] == 1
    assert out["get_ldim"] == 140 and out["set_epsrel_negative"] == 0 and out["default_detalg_is_hodlr"] == 1

    def ref(name, xi, m, key):
        return next(v[key] for v in ref_values[name] if v["xi"] == xi and v["m"] == m)

    want = {"pr_hodlr_xi1_m20": ref("pr_RbyL20_ldim140", 1.0, 20, "HODLR"),
            "pr_lu_xi1_m0": ref("pr_RbyL20_ldim140", 1.0, 0, "LU"),
            "pr_lu_xi1_m5": ref("pr_RbyL20_ldim140", 1.0, 5, "LU"),
            "drude_lu_xi3_m2": ref("drude_RbyL20_ldim140", 3.0, 2, "LU"),
            "drude_lu_xi12_m7": ref("drude_RbyL20_ldim140", 12.0, 7, "LU")}
    for k, w in want.items():
        assert abs(out[k] - w) <= 1e-10 * max(1.0, abs(w)), (k, out[k], w)
    mie = next(v for v in unit_vectors["test_mie_drude"]["cases"]
               if v["R"] == 1e-4 and v["L"] == 1e-4 and v["omegap_scaled"] == 5e4 and v["gamma_scaled"] == 1.0
               and v["xi"] == 1e-4 and v["l"] == 1)
    assert relx(out["mie_drude_lna"], mie["lna"]) < 1e-11 and relx(out["mie_drude_lnb"], mie["lnb"]) < 1e-11
    z = unit_vectors["test_logdetD0"]["m0_RbyL1000"]
    assert relx(out["xi0_EE"], z["EE"]) < 1e-10 and relx(out["xi0_MM"], z["MM"]) < 1e-10
