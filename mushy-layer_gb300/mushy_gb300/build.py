"""Builds the in-tree sm_103a library `_build/libmlgpu.so` with nvcc.

Translation units are compiled in parallel; the FP64 launcher unit is built
with --fmad=false so FP64 kernels keep the reference's unfused arithmetic.
Only one -gencode (sm_103a) is emitted.  No cmake, no torch extension
machinery: the library is a plain C-ABI shared object.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
CSRC = os.path.join(PKG_ROOT, "csrc")
BUILD = os.path.join(PKG_ROOT, "_build")
REPO = os.path.dirname(PKG_ROOT)
LIB = os.path.join(BUILD, "libmlgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "-lineinfo",
          "-I" + os.path.join(REPO, "include")]
UNITS = {
    "launch_f64.cu": ["--fmad=false"],
    "launch_f64_adj.cu": ["--fmad=false"],
    "launch_f64_nlc.cu": ["--fmad=false"],
    "launch_f32.cu": [],
    "launch_f32_fast.cu": [],
    "launch_f32_nlr.cu": [],
    "launch_f32_adj.cu": [],
    "capi.cu": ["--fmad=false"],
    "solver.cu": ["--fmad=false"],
    "capi_noalloc.cu": ["--fmad=false"],
}


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_mtime():
    m = 0.0
    for f in os.listdir(CSRC):
        m = max(m, os.path.getmtime(os.path.join(CSRC, f)))
    m = max(m, os.path.getmtime(os.path.join(REPO, "include", "mlgpu.h")))
    return m


def _compile(unit, extra):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, unit.replace(".cu", ".o"))
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (unit, " ".join(cmd), r.stderr))
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(*kv), UNITS.items()))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
