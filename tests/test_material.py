"""Tabulated materials (material_init / material_epsilonm1, the reference's material.c)
on the host, without a GPU: the library's reading of a synthetic optical-data file in the
reference's format against the unmodified reference's reading of the same file
(tests/golden/material_golden.json), and the reference's rejections."""
import ctypes as C
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FILE = os.path.join(HERE, "golden", "material_synthetic.txt")


@pytest.fixture(scope="module")
def lib():
    import importlib.util
    spec = importlib.util.spec_from_file_location("b", os.path.join(os.path.dirname(HERE), "caps_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    if not os.path.exists(b.LIB):
        pytest.skip("library not built")
    L = C.CDLL(b.LIB)
    L.material_init.restype = C.c_void_p
    L.material_init.argtypes = [C.c_char_p, C.c_double]
    L.material_free.argtypes = [C.c_void_p]
    L.material_epsilonm1.restype = C.c_double
    L.material_epsilonm1.argtypes = [C.c_double, C.c_void_p]
    L.material_get_extrapolation.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4
    return L


def test_material_matches_reference(lib):
    g = json.load(open(os.path.join(HERE, "golden", "material_golden.json")))
    m = lib.material_init(FILE.encode(), 11e-6)
    assert m
    ext = [C.c_double() for _ in range(4)]
    lib.material_get_extrapolation(m, *[C.byref(e) for e in ext])
    assert [e.value for e in ext] == g["extrapolation"]
    got = [lib.material_epsilonm1(x, m) for x in g["xi"]]
    assert got == g["epsm1"]
    lib.material_free(m)


def test_material_rejects(lib, tmp_path):
    assert not lib.material_init(str(tmp_path / "missing.txt").encode(), 1e-5)
    bad = tmp_path / "descending.txt"
    bad.write_text("# omegap_low = 9eV\n1e12 5.0\n2e12 4.0\n1.5e12 4.5\n")
    assert not lib.material_init(str(bad).encode(), 1e-5)
