// ref_host.cpp -- TEST INFRASTRUCTURE.  Runs the reference's own CUDA kernels
// (compiled unchanged into oracle/_ref/refkernels.fatbin by
// oracle/build_ref.py) the way the reference's host code launches them, on
// caller-supplied dense device arrays, so the tests can compare our
// restatements and our kernels with the reference's kernels on the same
// inputs.  Nothing here is product code; libcnncrf never links it.
//
// What the reference's launchers do and this file repeats:
//  - images live in pitched allocations (iu::ImageGpu is cudaMallocPitch'ed):
//    inputs are copied into pitched buffers and outputs copied back out;
//  - texture objects as bindTexture creates them (stereo/stereo.cu:84-157):
//    a pitch-2D resource of the element type, element reads, the given
//    address mode on both axes, normalised coordinates only in mirror mode,
//    linear filtering for 1- and 2-channel images unless point is asked for,
//    point filtering for 4-channel images;
//  - launch shapes: 32 x 32 blocks over the image (GPU_BLOCK_SIZE,
//    stereo/stereo.cu:28) for the image kernels, 480 threads per block over
//    the volume for the correlation (stereo/operators/stereocorrelation.cu:377-382);
//  - the TV loop of cuda::fuseTHuberQuadFit (stereo/stereo.cu:1133-1166) with
//    the textures of prepareFuseTTVL1 (stereo/stereo.cu:1097-1102).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ref_shim.cuh"

namespace {

thread_local std::string g_err;
cudaLibrary_t g_lib = nullptr;

int err(const char *what, cudaError_t e)
{
    g_err = std::string(what) + ": " + cudaGetErrorString(e);
    return 1;
}
#define CK(call)                                                                                                   \
    do {                                                                                                           \
        cudaError_t e__ = (call);                                                                                  \
        if (e__ != cudaSuccess) return err(#call, e__);                                                            \
    } while (0)

int kernel(const char *name, cudaKernel_t *k)
{
    if (!g_lib) {
        g_err = "module not loaded (ref_open)";
        return 1;
    }
    CK(cudaLibraryGetKernel(k, g_lib, name));
    return 0;
}

int launch(const char *name, dim3 grid, dim3 block, void **args)
{
    cudaKernel_t k;
    if (kernel(name, &k)) return 1;
    CK(cudaLaunchKernel((const void *)k, grid, block, args, 0, nullptr));
    CK(cudaGetLastError());
    CK(cudaDeviceSynchronize());
    return 0;
}

dim3 grid2d(int w, int h) { return dim3((w + 31) / 32, (h + 31) / 32); }

// a pitched image with its KernelData view; holds the allocation
template <class T> struct Pitched {
    T *p = nullptr;
    size_t pitch = 0;
    int w = 0, h = 0;
    ~Pitched()
    {
        if (p) cudaFree(p);
    }
    int alloc(int w_, int h_)
    {
        w = w_, h = h_;
        CK(cudaMallocPitch((void **)&p, &pitch, sizeof(T) * w, h));
        CK(cudaMemset2D(p, pitch, 0, sizeof(T) * w, h));
        return 0;
    }
    int from(const void *dense)
    {
        CK(cudaMemcpy2D(p, pitch, dense, sizeof(T) * w, sizeof(T) * w, h, cudaMemcpyDeviceToDevice));
        return 0;
    }
    int to(void *dense) const
    {
        CK(cudaMemcpy2D(dense, sizeof(T) * w, p, pitch, sizeof(T) * w, h, cudaMemcpyDeviceToDevice));
        return 0;
    }
    iu::PitchedKernelData<T> kd() const { return {p, w, h, (int)(pitch / sizeof(T))}; }
};

template <class T>
int bind(cudaTextureObject_t *tex, const Pitched<T> &m, cudaTextureAddressMode mode, cudaTextureFilterMode filter)
{
    cudaResourceDesc rd;
    std::memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypePitch2D;
    rd.res.pitch2D.devPtr = m.p;
    rd.res.pitch2D.pitchInBytes = m.pitch;
    rd.res.pitch2D.width = m.w;
    rd.res.pitch2D.height = m.h;
    rd.res.pitch2D.desc = cudaCreateChannelDesc<T>();
    cudaTextureDesc td;
    std::memset(&td, 0, sizeof(td));
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = mode == cudaAddressModeMirror;
    td.addressMode[0] = td.addressMode[1] = mode;
    td.filterMode = filter;
    CK(cudaCreateTextureObject(tex, &rd, &td, nullptr));
    return 0;
}

struct Tex {
    cudaTextureObject_t t = 0;
    ~Tex()
    {
        if (t) cudaDestroyTextureObject(t);
    }
};

iu::TensorGpu_32f::TensorKernelData tensor(float *p, int N, int C, int H, int W, bool nhwc)
{
    iu::TensorGpu_32f::TensorKernelData t;
    t.data_ = p;
    t.N = N, t.C = C, t.H = H, t.W = W;
    t.length_ = (unsigned)((long)N * C * H * W);
    t.nhwc = nhwc ? 1 : 0;
    return t;
}

} // namespace

extern "C" {

const char *ref_error() { return g_err.c_str(); }

int ref_open(const char *fatbin)
{
    if (g_lib) return 0;
    CK(cudaLibraryLoadFromFile(&g_lib, fatbin, nullptr, nullptr, 0, nullptr, nullptr, 0));
    return 0;
}

// cuda::forward on an NHWC output (stereo/operators/stereocorrelation.cu:358-408):
// out [N][H][W][D], im0 / im1 [N][C][H][W], disp: the D list entries as the
// reference stores them (-d, stereo/operators/stereocorrelation.cpp:83-85);
// interp: the kernel the reference picks when disparities[1] is not an integer
int ref_corr(float *out, float *im0, float *im1, float *disp, int N, int C, int H, int W, int D, int interp, int rect)
{
    auto o = tensor(out, N, D, H, W, true);
    auto a = tensor(im0, N, C, H, W, false), b = tensor(im1, N, C, H, W, false);
    iu::LinearDeviceMemory_32f_C1::KernelData d{disp, D};
    void *args[] = {&o, &a, &b, &d, &rect};
    const long n = (long)N * H * W * D;
    return launch(interp ? "ref_corr_nhwc_interp" : "ref_corr_nhwc", dim3((unsigned)std::ceil(n / 480.0f)),
                  dim3(480), args);
}

// cuda::calccostvolumecensus (stereo/stereo.cu:948-975): textures clamp / linear
int ref_census(float *vol, const float *I1, const float *I2, int W, int H, int fs, float dmin, float dstep, int depth,
               float lam)
{
    Pitched<float> a, b;
    if (a.alloc(W, H) || b.alloc(W, H) || a.from(I1) || b.from(I2)) return 1;
    Tex t1, t2;
    if (bind(&t1.t, a, cudaAddressModeClamp, cudaFilterModeLinear) ||
        bind(&t2.t, b, cudaAddressModeClamp, cudaFilterModeLinear))
        return 1;
    iu::LinearDeviceMemory_32f_C1::KernelData v{vol, W * H * depth};
    void *args[] = {&v, &t1.t, &t2.t, &dmin, &dstep, &fs, &fs, &lam, &W, &H, &depth};
    return launch("ref_census", grid2d(W, H), dim3(32, 32), args);
}

// cuda::computeArgmin (stereo/stereo.cu:977-995)
int ref_argmin(float *out, float *vol, int W, int H, int depth, float dmin, float dstep)
{
    Pitched<float> o;
    if (o.alloc(W, H)) return 1;
    auto kd = o.kd();
    iu::LinearDeviceMemory_32f_C1::KernelData v{vol, W * H * depth};
    void *args[] = {&kd, &v, &depth, &dmin, &dstep};
    if (launch("ref_argmin", grid2d(W, H), dim3(32, 32), args)) return 1;
    return o.to(out);
}

// do_fitting_kernel on a 3-label NHWC volume [H][W][3] -> qf [H][W][2]
int ref_fit(float *qf, float *vol3, int W, int H, float step, float lam, int do_abs)
{
    Pitched<float2> o;
    if (o.alloc(W, H)) return 1;
    auto kd = o.kd();
    auto v = tensor(vol3, 1, 3, H, W, true);
    bool da = do_abs != 0;
    void *args[] = {&kd, &v, &step, &lam, &da};
    if (launch("ref_fit", grid2d(W, H), dim3(32, 32), args)) return 1;
    return o.to(qf);
}

// the TV loop of cuda::fuseTHuberQuadFit for one warp (stereo/stereo.cu:1133-1166):
// p = q = 0, tau = sigma = 1/sqrt(8), `iters` x (u_ = u; primal; dual).
// u: in / out; u_, p, q: out; wx, wy: the edge weights
int ref_tv(float *u, float *u_out, const float *u0, const float *qf, const float *wx, const float *wy, float *p_out,
           float *q_out, int W, int H, float C, float step, int iters)
{
    Pitched<float> pu, pu_, pu0, pwx, pwy;
    Pitched<float2> pqf, pp, pq;
    if (pu.alloc(W, H) || pu_.alloc(W, H) || pu0.alloc(W, H) || pwx.alloc(W, H) || pwy.alloc(W, H) ||
        pqf.alloc(W, H) || pp.alloc(W, H) || pq.alloc(W, H))
        return 1;
    if (pu.from(u) || pu0.from(u0) || pwx.from(wx) || pwy.from(wy) || pqf.from(qf)) return 1;
    Tex tu_, tp, tq;
    if (bind(&tu_.t, pu_, cudaAddressModeClamp, cudaFilterModePoint) ||
        bind(&tp.t, pp, cudaAddressModeClamp, cudaFilterModeLinear) ||
        bind(&tq.t, pq, cudaAddressModeClamp, cudaFilterModeLinear))
        return 1;
    float L = sqrt(8);
    float tau = 1 / L, sigma = 1 / L;
    auto ku = pu.kd(), ku_ = pu_.kd(), ku0 = pu0.kd(), kwx = pwx.kd(), kwy = pwy.kd();
    auto kqf = pqf.kd(), kp = pp.kd(), kq = pq.kd();
    for (int it = 0; it < iters; ++it) {
        CK(cudaMemcpy2D(pu_.p, pu_.pitch, pu.p, pu.pitch, sizeof(float) * W, H, cudaMemcpyDeviceToDevice));
        void *pa[] = {&ku, &ku_, &ku0, &kqf, &tp.t, &tq.t, &tau, &step};
        if (launch("ref_primal", grid2d(W, H), dim3(32, 32), pa)) return 1;
        void *da[] = {&kp, &kq, &kwx, &kwy, &tu_.t, &sigma, &C};
        if (launch("ref_dual", grid2d(W, H), dim3(32, 32), da)) return 1;
    }
    if (pu.to(u) || pu_.to(u_out) || pp.to(p_out) || pq.to(q_out)) return 1;
    return 0;
}

// cuda::leftRightCheck (stereo/stereo.cu:1198-1220): textures clamp / linear
int ref_lrcheck(float *out, const float *left, const float *right, int W, int H, float th)
{
    Pitched<float> o, l, r;
    if (o.alloc(W, H) || l.alloc(W, H) || r.alloc(W, H) || l.from(left) || r.from(right)) return 1;
    Tex tl, tr;
    if (bind(&tl.t, l, cudaAddressModeClamp, cudaFilterModeLinear) ||
        bind(&tr.t, r, cudaAddressModeClamp, cudaFilterModeLinear))
        return 1;
    auto kd = o.kd();
    void *args[] = {&kd, &tl.t, &tr.t, &th};
    if (launch("ref_lrcheck", grid2d(W, H), dim3(32, 32), args)) return 1;
    return o.to(out);
}

// warp_image_kernel on an RGBA image, texture clamp / point (stereo/stereo.cu:1138,1150)
int ref_warp_c4(float *out, const float *disp, const float *in, int W, int H)
{
    Pitched<float4> o, i;
    Pitched<float> d;
    if (o.alloc(W, H) || i.alloc(W, H) || d.alloc(W, H) || i.from(in) || d.from(disp)) return 1;
    Tex t;
    if (bind(&t.t, i, cudaAddressModeClamp, cudaFilterModePoint)) return 1;
    auto ko = o.kd();
    auto kd = d.kd();
    void *args[] = {&ko, &kd, &t.t};
    if (launch("ref_warp_c4", grid2d(W, H), dim3(32, 32), args)) return 1;
    return o.to(out);
}

// cuda::remapSolution (stereo/stereo.cu:1229-1246)
int ref_remap(float *out, const int *labels, int W, int H, float dmin, float dstep)
{
    Pitched<float> o;
    Pitched<int> l;
    if (o.alloc(W, H) || l.alloc(W, H) || l.from(labels)) return 1;
    auto ko = o.kd();
    auto kl = l.kd();
    void *args[] = {&ko, &kl, &dmin, &dstep};
    if (launch("ref_remap", grid2d(W, H), dim3(32, 32), args)) return 1;
    return o.to(out);
}

// cuda::rgb2gray (stereo/stereo.cu:1248-1259)
int ref_rgb2gray(float *gray, const float *rgba, int W, int H)
{
    Pitched<float4> i;
    Pitched<float> o;
    if (i.alloc(W, H) || o.alloc(W, H) || i.from(rgba)) return 1;
    auto ki = i.kd();
    auto ko = o.kd();
    void *args[] = {&ki, &ko};
    if (launch("ref_rgb2gray", grid2d(W, H), dim3(32, 32), args)) return 1;
    return o.to(gray);
}

// cuda::padColorImage (stereo/stereo.cu:1022-1044): texture mirror (normalised coordinates) / point
int ref_pad_color(float *out, const float *in, int W, int H, int pad)
{
    Pitched<float4> i, o;
    if (i.alloc(W, H) || o.alloc(W + 2 * pad, H + 2 * pad) || i.from(in)) return 1;
    Tex t;
    if (bind(&t.t, i, cudaAddressModeMirror, cudaFilterModePoint)) return 1;
    auto ko = o.kd();
    void *args[] = {&ko, &t.t, &pad};
    if (launch("ref_pad_color", grid2d(W + 2 * pad, H + 2 * pad), dim3(32, 32), args)) return 1;
    return o.to(out);
}

// cuda::fuseQuadFitDirect (stereo/stereo.cu:1172-1194) on the volume get_C1()
// as Stereo passes it (H x W x D, viewed {W, H, D} by permute_dims({1, 2, 0}),
// stereo/stereo.cpp:406-410): u in / out
int ref_quadfit_direct(float *u, float *vol, int W, int H, int D, float dmin, float dstep)
{
    Pitched<float> pu;
    Pitched<float2> qf;
    if (pu.alloc(W, H) || qf.alloc(W, H) || pu.from(u)) return 1;
    kernel::ndarray_ref<float, 3> v;
    v.data_ = vol;
    v.size_[0] = W, v.size_[1] = H, v.size_[2] = D;
    v.stride_[0] = D, v.stride_[1] = (long)D * W, v.stride_[2] = 1;
    auto kq = qf.kd();
    auto ku = pu.kd();
    float lam = 1.f;
    void *fa[] = {&kq, &ku, &v, &dmin, &dstep, &lam};
    if (launch("ref_fit_volume", grid2d(W, H), dim3(32, 32), fa)) return 1;
    void *aa[] = {&ku, &kq};
    if (launch("ref_argmin_volume", grid2d(W, H), dim3(32, 32), aa)) return 1;
    return pu.to(u);
}

} // extern "C"
