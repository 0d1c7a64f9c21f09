"""Build recipe of libcnncrf.so (the product): nvcc for the CUDA kernels
(sm_103a only), g++ for the host code, linked against the shared CUDA runtime.

Kernels whose results must equal the CPU oracle bit for bit are compiled with
--fmad=false (every fused multiply-add in them is written out explicitly);
the tensor-core files keep the default contraction.  Objects are built in
parallel into _build/, the library lands in cnncrf/libcnncrf.so (in tree).
"""
import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "cnncrf", "libcnncrf.so")
INC = os.path.join(HERE, "..", "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# kernels that must match the oracle bit for bit
EXACT = {"k_front.cu", "k_conv_simt.cu", "k_corr.cu", "k_crf.cu", "k_crf_r4.cu", "k_misc.cu", "k_census.cu", "k_tv.cu"}


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cu, cpp


def _headers_hash():
    h = hashlib.sha1()
    for d in (CSRC, INC):
        for f in sorted(os.listdir(d)):
            if f.endswith((".h", ".cuh")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode() + fh.read())
    return h.hexdigest()


def _cmd(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if src.endswith(".cu"):
        cmd = [NVCC] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                               "-I" + INC, "-c", path, "-o", obj]
        if src in EXACT:
            cmd.insert(1, "--fmad=false")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
               "-I" + os.path.join(CUDA_HOME, "include"), "-I" + INC, "-c", path, "-o", obj]
    return cmd, path, obj


def build(force=False, verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp = _sources()
    stamp = os.path.join(BUILD, "headers.sha1")
    hh = _headers_hash()
    if not force and os.path.exists(stamp) and open(stamp).read() != hh:
        force = True
    work = []
    for src in cu + cpp:
        cmd, path, obj = _cmd(src)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(path):
            work.append(cmd)
    objs = [_cmd(s)[2] for s in cu + cpp]

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return r.stderr

    jobs = jobs or min(16, os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        for err in ex.map(run, work):
            if verbose and err:
                print(err, file=sys.stderr)
    if work or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + \
              ["-Xlinker", "-rpath=" + os.path.join(CUDA_HOME, "lib64")]
        run(cmd)
        os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(hh)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
