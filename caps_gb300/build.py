"""Build the GB300 CaPS library (CUDA, sm_103a) and the CPU oracle.

The library is compiled in-tree into caps_gb300/_build/libcaps_gb300.so with
one nvcc process per translation unit (run in parallel) and a final link.
The oracle (test infrastructure) goes to oracle/_build/liboracle.so.  When the
CaPS source tree is available (CAPS_REFERENCE_SRC or ../reference next to the
checkout), its unmodified library is also built into oracle/_ref/ as a second
parity reference.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "caps_gb300", "csrc")
BUILD = os.path.join(ROOT, "caps_gb300", "_build")
LIB = os.path.join(BUILD, "libcaps_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

SOURCES = ["libcaps.cu", "assemble.cu", "cholesky.cu", "xi0.cu", "noalloc.cu", "mixed.cu", "mlp.cu", "elem_ff.cu", "itab_ff.cu", "tzero.cu", "material.cu", "square.cu", "capc.cu", "hodlr.cu", "sweep.cu"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("command failed: " + " ".join(cmd))
    return r


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(force=False):
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "libcaps.h"))
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    objs = []
    jobs = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([_nvcc(), *NVCC_FLAGS, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        _run([_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", LIB, *objs])
    return LIB


def build_oracle(force=False):
    os.makedirs(os.path.dirname(ORACLE_LIB), exist_ok=True)
    src = os.path.join(ORACLE_DIR, "caps_oracle.c")
    hdr = os.path.join(ORACLE_DIR, "caps_oracle.h")
    if force or _stale(ORACLE_LIB, [src, hdr]):
        _run(["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-D_GNU_SOURCE", "-o", ORACLE_LIB, src, "-lm", "-lpthread"])
    return ORACLE_LIB


def reference_source():
    cand = [os.environ.get("CAPS_REFERENCE_SRC", ""), os.path.join(os.path.dirname(ROOT), "reference")]
    for c in cand:
        if c and os.path.exists(os.path.join(c, "src", "libcaps.c")):
            return c
    return None


def build_reference():
    ref = reference_source()
    if ref is None:
        return None
    _run(["make", "-s", "-f", os.path.join(ORACLE_DIR, "Makefile.ref"), "REF=" + ref, "-j8", "-C", ROOT])
    return os.path.join(ORACLE_DIR, "_ref", "libcaps_ref.so")


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv))
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference())
