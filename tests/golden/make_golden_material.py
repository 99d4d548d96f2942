"""A synthetic optical-data file in the reference's material format, and the unmodified
reference library's view of it (oracle/_ref/libcaps_ref.so, material.c): eps(i xi)-1 at
interior, tabulated, boundary and extrapolated frequencies, and the extrapolation
parameters.  The data are made up here (Drude metal plus one Lorentz oscillator), not
taken from any measured material.

    python tests/golden/make_golden_material.py   # writes material_synthetic.txt, material_golden.json
"""
import ctypes as C
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
HBAR_EV = 6.582119514e-16
FILE = os.path.join(HERE, "material_synthetic.txt")


def eps(xi):
    wp, ga = 8.7 / HBAR_EV, 0.04 / HBAR_EV
    w0, wl, gl = 3.1 / HBAR_EV, 4.0 / HBAR_EV, 0.8 / HBAR_EV
    return 1 + wp * wp / (xi * (xi + ga)) + wl * wl / (w0 * w0 + xi * xi + gl * xi)


def write_file():
    lines = ["# synthetic test material: Drude metal plus one Lorentz oscillator",
             "# Drude parameters for low frequencies",
             "#\tomegap_low = 8.7eV", "# gamma_low  = 0.04eV", "#",
             "# omegap_high = 12.25 eV", "# gamma_high=1.5eV", "# xi in rad/s   epsilon(i*xi)"]
    xs = [10 ** (11.2 + 7.0 * k / 400) for k in range(401)]
    for k, x in enumerate(xs):
        sep = "\t" if k % 3 == 0 else ("   " if k % 3 == 1 else " ")
        xs_txt = ("%.16E" % x) if k % 2 else ("%.4f" % x)
        lines.append("  " + xs_txt + sep + ("%.15g" % eps(x)) + ("  " if k % 5 == 0 else ""))
    open(FILE, "w").write("\n".join(lines) + "\n")


def main():
    write_file()
    lib = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libcaps_ref.so"))
    lib.material_init.restype = C.c_void_p
    lib.material_init.argtypes = [C.c_char_p, C.c_double]
    lib.material_epsilonm1.restype = C.c_double
    lib.material_epsilonm1.argtypes = [C.c_double, C.c_void_p]
    lib.material_get_extrapolation.argtypes = [C.c_void_p] + [C.POINTER(C.c_double)] * 4
    m = lib.material_init(FILE.encode(), 11e-6)
    assert m
    ext = [C.c_double() for _ in range(4)]
    lib.material_get_extrapolation(m, *[C.byref(e) for e in ext])
    probes = [10 ** (10.0 + 9.5 * k / 997) for k in range(998)]
    with open(FILE) as f:
        nodes = [float(l.split()[0]) for l in f if l.strip() and not l.strip().startswith("#")]
    probes += nodes[:5] + nodes[-5:] + [nodes[0] * (1 - 1e-15), nodes[-1] * (1 + 1e-15)]
    out = dict(source="oracle/_ref/libcaps_ref.so material_init/material_epsilonm1 on tests/golden/material_synthetic.txt",
               extrapolation=[e.value for e in ext], xi=probes, epsm1=[lib.material_epsilonm1(x, m) for x in probes])
    json.dump(out, open(os.path.join(HERE, "material_golden.json"), "w"), indent=1)
    print(len(probes), out["extrapolation"])


if __name__ == "__main__":
    main()
