"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle.cpp into oracle/_build/liboracle.so with IEEE evaluation
order kept (-ffp-contract=off, no fast-math) so FP64 results can be compared
bit for bit with the sm_103a kernels, and OpenMP for the timed CPU baseline.
The same flags are used on x86-64 and aarch64 (no -march=native).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "oracle.cpp")
HDR = os.path.join(HERE, "..", "include", "mlgpu.h")


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR))
        if os.path.getmtime(LIB) >= newest:
            return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-o", tmp, SRC]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
