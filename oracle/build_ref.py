"""Build recipe of the reference-kernel module (TEST INFRASTRUCTURE).

Compiles the reference's own CUDA kernels for the hot path's non-CRF stages,
unchanged, from the reference tree into a device-code module,
oracle/_ref/refkernels.fatbin (sm_103a).  The tests run them as a second
oracle through oracle/ref_host.cpp.  The reference's full build cannot run
here (its imageutilities, SlackProp and cnpy submodules are empty, and
Boost, OpenCV and png++ are absent), but these kernels depend only on the
iu:: container accessors, helper math and ndarray_ref, which
oracle/ref_shim.cuh restates.

The kernels' definitions are cut out of the reference files by name (every
overload; brace-matched) into oracle/_ref/refkernels.cu, which is never
committed (oracle/_ref/ is git-ignored), behind the shim header.  Their
`__global__` is read as `__device__` there, and one extern "C" __global__
wrapper per kernel calls it, so the module exports unmangled names with the
same launch semantics (blockIdx / threadIdx are the wrapper's).  Flags follow
the reference's release build (cmake/compiler_settings.cmake.txt:4,9: -O2
-lineinfo -DNDEBUG, default FMA contraction and IEEE division), without its
-keep / -src-in-ptx.

usage: python oracle/build_ref.py [REFERENCE_ROOT]
(REFERENCE_ROOT defaults to $CNNCRF_REFERENCE; the module is only built where
the reference tree exists; the GPU machines use the prebuilt file.)
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
FATBIN = os.path.join(OUT_DIR, "refkernels.fatbin")
GEN = os.path.join(OUT_DIR, "refkernels.cu")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")

# (file, definitions to cut out: the start of each signature; every match is taken)
PIECES = [
    ("stereo/operators/stereocorrelation.cu", [
        "__device__ float dLinearInterpolation1D(",
        "__global__ void kCorrelation_NHWC_interpolation(",
        "__global__ void kCorrelation_NHWC(",
    ]),
    ("stereo/stereo.cu", [
        "__global__ void cost_vol_census_kernel(",
        "__global__ void arg_min_kernel(",
        "__global__ void do_fitting_kernel(",
        "__global__ void ttvqf_primal_kernel(",
        "__device__ inline float2 sign(",
        "__device__ inline float sign(",
        "__device__ inline float2 max(",
        "__device__ inline float prox_p(",
        "__device__ inline float2 prox_p(",
        "__device__ inline float4 prox_p(",
        "__global__ void thuberqf_dual_kernel(",
        "__global__ void leftrightcheck_kernel(",
        "__global__ void warp_image_kernel(",
        "__global__ void remapsolution_kernel(",
        "__global__ void rgb_to_gray_kernel(",
        "__global__ void padding_color_kernel(",
        "__global__ void do_fitting_kernel_volume(",
        "__global__ void do_argmin_kernel_volume(",
    ]),
]

# exported entry points: name, parameter list, the reference kernel it calls
WRAPPERS = [
    ("ref_corr_nhwc", "iu::TensorGpu_32f::TensorKernelData o, iu::TensorGpu_32f::TensorKernelData a, "
                      "iu::TensorGpu_32f::TensorKernelData b, iu::LinearDeviceMemory_32f_C1::KernelData d, int r",
     "kCorrelation_NHWC(o, a, b, d, r)"),
    ("ref_corr_nhwc_interp", "iu::TensorGpu_32f::TensorKernelData o, iu::TensorGpu_32f::TensorKernelData a, "
                             "iu::TensorGpu_32f::TensorKernelData b, iu::LinearDeviceMemory_32f_C1::KernelData d, "
                             "int r",
     "kCorrelation_NHWC_interpolation(o, a, b, d, r)"),
    ("ref_census", "iu::LinearDeviceMemory_32f_C1::KernelData v, cudaTextureObject_t t1, cudaTextureObject_t t2, "
                   "float dmin, float dstep, int fw, int fh, float lam, int w, int h, int depth",
     "cost_vol_census_kernel(v, t1, t2, dmin, dstep, fw, fh, lam, w, h, depth)"),
    ("ref_argmin", "iu::ImageGpu_32f_C1::KernelData out, iu::LinearDeviceMemory_32f_C1::KernelData v, int depth, "
                   "float dmin, float dstep",
     "arg_min_kernel(out, v, depth, dmin, dstep)"),
    ("ref_fit", "iu::ImageGpu_32f_C2::KernelData out, iu::TensorGpu_32f::TensorKernelData v, float step, "
                "float lam, bool do_abs",
     "do_fitting_kernel(out, v, step, lam, do_abs)"),
    ("ref_primal", "iu::ImageGpu_32f_C1::KernelData u, iu::ImageGpu_32f_C1::KernelData u_, "
                   "iu::ImageGpu_32f_C1::KernelData u0, iu::ImageGpu_32f_C2::KernelData qf, "
                   "cudaTextureObject_t tp, cudaTextureObject_t tq, float tau, float step",
     "ttvqf_primal_kernel(u, u_, u0, qf, tp, tq, tau, step)"),
    ("ref_dual", "iu::ImageGpu_32f_C2::KernelData p, iu::ImageGpu_32f_C2::KernelData q, "
                 "iu::ImageGpu_32f_C1::KernelData wx, iu::ImageGpu_32f_C1::KernelData wy, cudaTextureObject_t tu, "
                 "float sigma, float C",
     "thuberqf_dual_kernel(p, q, wx, wy, tu, sigma, C)"),
    ("ref_lrcheck", "iu::ImageGpu_32f_C1::KernelData out, cudaTextureObject_t tl, cudaTextureObject_t tr, float th",
     "leftrightcheck_kernel(out, tl, tr, th)"),
    ("ref_warp_c4", "iu::ImageGpu_32f_C4::KernelData out, iu::ImageGpu_32f_C1::KernelData disp, "
                    "cudaTextureObject_t tin",
     "warp_image_kernel(out, disp, tin)"),
    ("ref_remap", "iu::ImageGpu_32f_C1::KernelData out, iu::ImageGpu_32s_C1::KernelData in, float dmin, float dstep",
     "remapsolution_kernel(out, in, dmin, dstep)"),
    ("ref_rgb2gray", "iu::ImageGpu_32f_C4::KernelData rgb, iu::ImageGpu_32f_C1::KernelData gray",
     "rgb_to_gray_kernel(rgb, gray)"),
    ("ref_pad_color", "iu::ImageGpu_32f_C4::KernelData out, cudaTextureObject_t tin, int padval",
     "padding_color_kernel(out, tin, padval)"),
    ("ref_fit_volume", "iu::ImageGpu_32f_C2::KernelData out, iu::ImageGpu_32f_C1::KernelData sp, "
                       "kernel::ndarray_ref<float, 3> v, float dmin, float dstep, float lam",
     "do_fitting_kernel_volume(out, sp, v, dmin, dstep, lam)"),
    ("ref_argmin_volume", "iu::ImageGpu_32f_C1::KernelData io, iu::ImageGpu_32f_C2::KernelData qf",
     "do_argmin_kernel_volume(io, qf)"),
]


def _body_end(text, i):
    """Index just past the brace that closes the first '{' at or after i,
    skipping comments and string / character literals."""
    depth, n, started = 0, len(text), False
    while i < n:
        c = text[i]
        if text.startswith("//", i):
            i = text.index("\n", i)
            continue
        if text.startswith("/*", i):
            i = text.index("*/", i) + 2
            continue
        if c in "\"'":
            j = i + 1
            while text[j] != c:
                j += 2 if text[j] == "\\" else 1
            i = j + 1
            continue
        if c == "{":
            depth += 1
            started = True
        elif c == "}":
            depth -= 1
            if started and depth == 0:
                return i + 1
        i += 1
    raise ValueError("unbalanced braces")


def extract(ref_root):
    out = []
    for rel, starts in PIECES:
        path = os.path.join(ref_root, rel)
        with open(path) as f:
            text = f.read()
        for s in starts:
            hits = [m.start() for m in re.finditer(re.escape(s), text)]
            if not hits:
                raise ValueError("%s: no definition starting %r" % (rel, s))
            for h in hits:
                line = text.count("\n", 0, h) + 1
                end = _body_end(text, h)
                out.append('#line %d "%s"\n%s\n' % (line, rel, text[h:end]))
    return out


def generate(ref_root):
    parts = ["// generated by oracle/build_ref.py from the reference tree; not committed\n",
             '#include "ref_shim.cuh"\n',
             '#pragma push_macro("__global__")\n#undef __global__\n#define __global__ __device__\n']
    parts += extract(ref_root)
    parts.append('#pragma pop_macro("__global__")\n#line 1 "refkernels_wrappers"\n')
    for name, params, call in WRAPPERS:
        parts.append('extern "C" __global__ void %s(%s) { %s; }\n' % (name, params, call))
    return "".join(parts)


def build(ref_root=None, force=False, verbose=False):
    ref_root = ref_root or os.environ.get("CNNCRF_REFERENCE")
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "stereo")):
        return None  # no reference tree here: use the prebuilt module if present
    srcs = [os.path.join(ref_root, rel) for rel, _ in PIECES] + [os.path.join(HERE, "ref_shim.cuh"), __file__]
    if not force and os.path.exists(FATBIN) and all(os.path.getmtime(s) <= os.path.getmtime(FATBIN) for s in srcs):
        return FATBIN
    os.makedirs(OUT_DIR, exist_ok=True)
    with open(GEN, "w") as f:
        f.write(generate(ref_root))
    tmp = FATBIN + ".tmp"
    cmd = [NVCC, "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-lineinfo", "-DNDEBUG",
           "-std=c++17", "-I" + HERE, GEN, "-o", tmp]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, FATBIN)
    return FATBIN


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else None
    print(build(root, force=True, verbose=True))
