"""Build the engine library (libcrvgpu.so) in-tree with nvcc for sm_103a.

The translation units compile in parallel: the engine/C-ABI unit, the FP64 kernels and the lookup-table substep unit
(both built with -fmad=false so every FP64 operation rounds exactly as written: bit-exact with the CPU oracle), the
FP32-mixed kernels and the allocation-free pulse-fit entry point.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(PKG))
CSRC = os.path.join(os.path.dirname(PKG), "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIB_DIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIB_DIR, "libcrvgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
UNITS = {
    "crv_engine.cu": [],
    "crv_kernels_f64.cu": ["-fmad=false"],
    "crv_kernels_f32.cu": [],
    "crv_static.cu": [],
    "crv_lookup.cu": ["-fmad=false"],
    "crv_tables.cpp": [],                 # host code (lookup-table file reader)
    "crv_rootio.cpp": [],                 # host code (LZ4 / XXH64 of ROOT step-table baskets)
}


def nvcc():
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(n):
        raise RuntimeError("nvcc not found: the CRV engine needs the CUDA toolkit to build")
    return n


def sources():
    out = []
    for d in (CSRC, INCLUDE):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cu", ".cpp", ".cuh", ".h", ".inc")):
                out.append(os.path.join(d, f))
    return out


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in sources())


def build(force=False, verbose=False, extra=None):
    """Compile libcrvgpu.so (skipped when up to date).  Returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(LIB_DIR, exist_ok=True)
    obj_dir = os.path.join(LIB_DIR, f"obj_{os.getpid()}")
    os.makedirs(obj_dir, exist_ok=True)
    common = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE,
              "-I", CSRC, "--expt-relaxed-constexpr"] + list(extra or [])

    def one(item):
        src, flags = item
        obj = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
        cmd = common + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr, file=sys.stderr)
        return obj

    tmp = LIB + f".{os.getpid()}.tmp"
    try:
        with ThreadPoolExecutor(len(UNITS)) as ex:
            objs = list(ex.map(one, UNITS.items()))
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    finally:                                    # objects and a partial link never outlive the call
        shutil.rmtree(obj_dir, ignore_errors=True)
        if os.path.exists(tmp):
            os.remove(tmp)
    return LIB


if __name__ == "__main__":
    v = "-v" in sys.argv
    print(build(force=True, verbose=v, extra=["-Xptxas", "-v"] if v else None))
