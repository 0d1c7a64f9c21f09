"""Build recipe of the CPU oracle (TEST INFRASTRUCTURE, see cnncrf_oracle.h).

Compiles oracle/cnncrf_oracle.cpp into oracle/_build/liboracle.so with g++ and
OpenMP, and the launcher of the reference's own kernels (oracle/ref_host.cpp)
into oracle/_build/libref_host.so against the CUDA runtime; the reference's
kernel module itself is built by oracle/build_ref.py where the reference tree
exists.  -ffp-contract=off keeps a*b+c from being fused behind our back: the
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


REF_HOST_SRC = os.path.join(HERE, "ref_host.cpp")
REF_HOST_LIB = os.path.join(OUT_DIR, "libref_host.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_ref_host(force=False, verbose=False):
    deps = [REF_HOST_SRC, os.path.join(HERE, "ref_shim.cuh")]
    if not force and os.path.exists(REF_HOST_LIB) and \
            all(os.path.getmtime(d) <= os.path.getmtime(REF_HOST_LIB) for d in deps):
        return REF_HOST_LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = REF_HOST_LIB + ".tmp"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I" + os.path.join(CUDA_HOME, "include"), "-I" + HERE,
           REF_HOST_SRC, "-o", tmp, "-L" + os.path.join(CUDA_HOME, "lib64"), "-lcudart",
           "-Wl,-rpath," + os.path.join(CUDA_HOME, "lib64")]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_HOST_LIB)
    return REF_HOST_LIB


def build(force=False, verbose=False):
    build_ref_host(force, verbose)
    from oracle import build_ref  # the reference's kernels, where the reference tree is present
    build_ref.build(os.environ.get("CNNCRF_REFERENCE") or ("/root/reference" if os.path.isdir("/root/reference")
                                                           else None))
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
