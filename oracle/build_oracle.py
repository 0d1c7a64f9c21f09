"""Build recipe of the CPU oracle (TEST INFRASTRUCTURE, see cnncrf_oracle.h).

Compiles oracle/cnncrf_oracle.cpp into oracle/_build/liboracle.so with g++ and
OpenMP.  -ffp-contract=off keeps a*b+c from being fused behind our back: the
float build must follow the explicit operation order of the GPU FP32 path.
On x86-64 -mfma makes fmaf() a single instruction (aarch64 always has it).
"""
import os
import platform
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "cnncrf_oracle.cpp")


def needs_build():
    if not os.path.exists(LIB):
        return True
    deps = [SRC, os.path.join(HERE, "cnncrf_oracle.h"),
            os.path.join(HERE, "..", "include", "cnncrf_fmath.h"),
            os.path.join(HERE, "..", "include", "cnncrf_xavier.h")]
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    flags = ["-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
             "-fPIC", "-shared"]
    if platform.machine() in ("x86_64", "AMD64"):
        flags.append("-mfma")
    tmp = LIB + ".tmp"
    cmd = ["g++"] + flags + [SRC, "-o", tmp]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
