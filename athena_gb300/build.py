"""Build the CUDA library libathgpu.so in-tree (sm_103a, nvcc, no CMake).

``python -m athena_gb300.build`` or ``athena_gb300.build.build()``.  Translation units
compile in parallel; the FP64 stage unit is compiled with ``-fmad=false`` so that no FMA
contraction changes its rounding relative to the reference's FP64 build.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libathgpu.so")
OBJDIR = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]

UNITS = {
    "api.cu": ["-fmad=false"],
    "stage_fp64.cu": ["-fmad=false"],
    # FP32 path: FMA contraction and the fast (approximate) FP32 divide and square root
    "stage_fp32.cu": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"],
    "noalloc.cu": ["-fmad=false"],
    # learned con2prim: the FP64 polish keeps the reference's rounding (no contraction)
    "sr_learned.cu": ["-fmad=false"],
    "selftest.cu": ["-fmad=false"],
    "history.cu": ["-fmad=false"],
    # div B diagnostic (the reference's per-cell arithmetic) and run statistics
    "diagnostics.cu": ["-fmad=false"],
    # per-operator entry points on one MeshBlock (FP64, the reference's rounding)
    "operators.cu": ["-fmad=false"],
    # host planner of the multi-level stage
    "ml_plan.cu": ["-fmad=false"],
    # adaptive refinement: refinement measure and regrid (FP64 restriction/prolongation)
    "regrid.cu": ["-fmad=false"],
    # adaptive refinement, host side: block tree, neighbour lists, coordinates, flags
    "amr_host.cu": ["-fmad=false"],
}


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "athena_gb300.h")]


def build(force=False, verbose=False):
    newest = max(os.path.getmtime(p) for p in _deps())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    cc = nvcc()

    def compile_unit(item):
        src, flags = item
        obj = os.path.join(OBJDIR, src.replace(".cu", ".o"))
        cmd = [cc] + ARCH + BASE + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s" % (src, r.stderr[-6000:]))
        return obj, r.stderr

    with ThreadPoolExecutor(len(UNITS)) as ex:
        results = list(ex.map(compile_unit, UNITS.items()))
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
