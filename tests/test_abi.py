"""The C-ABI library loads without a GPU and exports every function declared in
include/*.h.  No compute call is made here."""
import ctypes as C
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    inc = os.path.join(ROOT, "include")
    for h in sorted(os.listdir(inc)):
        if not h.endswith(".h"):
            continue
        src = re.sub(r"/\*.*?\*/", "", open(os.path.join(inc, h)).read(), flags=re.S)
        names.update(re.findall(r"^[A-Za-z_][\w \*]*?\b((?:caps|bessel|material)_\w+)\s*\(", src, flags=re.M))
    return sorted(names)


def test_header_parsed():
    names = declared_functions()
    assert "caps_logdetD" in names and "caps_logdetD_batch" in names and len(names) >= 38
    assert "caps_capc_energy_T0" in names and "bessel_logKn" in names and "material_epsilonm1" in names


def test_library_exports_all():
    import caps_gb300
    lib = C.CDLL(caps_gb300.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_host_helpers_match_oracle():
    import caps_gb300 as cg
    from oracle import binding as ob
    for l1, l2, m in [(1, 1, 0), (5, 9, 3), (300, 1200, 200), (2000, 2100, 1000)]:
        assert abs(cg.lib.caps_lnLambda(l1, l2, m) - ob.lib.oracle_lnLambda(l1, l2, m)) < 1e-12
    c = cg.Caps(150e-6, 1e-6, ldim=1050)
    for m in (0, 1, 10, 68, 69, 200, 400):
        assert c.lminmax(m)[0] == ob.lib.oracle_lmin(1e-6 / 150e-6, 1050, m)
    assert c.ldim == 1050
    d = cg.Caps(20e-6, 1e-6)
    assert d.ldim == 101  # ceil(max(20, 5/(L/R))) in floating point, as the reference computes it
    assert cg.lib.caps_init(-1.0, 1.0) is None
    assert cg.lib.caps_set_ldim(d._h, 0) == 0


def test_fresnel_reference_vectors(unit_vectors):
    """the host helper caps_fresnel against all 3430 asserts of the reference's
    src/tests/test_fresnel.c (Drude metals, relative tolerance 2e-15)"""
    import caps_gb300 as cg
    from conftest import relx
    t = unit_vectors["test_fresnel"]
    c = cg.Caps(t["R"], t["L"])
    mat, bad = None, []
    for v in t["cases"]:
        if (v["omegap_eV"], v["gamma_eV"]) != mat:
            mat = (v["omegap_eV"], v["gamma_eV"])
            c.set_drude(*mat)
        te, tm = c.fresnel(v["xi"], v["k"])
        if not (relx(te, v["rTE"]) < t["tolerance"] and relx(tm, v["rTM"]) < t["tolerance"]):
            bad.append((v, te, tm))
    assert len(t["cases"]) == 1715 and not bad, (len(bad), bad[:3])
