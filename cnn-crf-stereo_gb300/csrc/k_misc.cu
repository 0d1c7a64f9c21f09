// k_misc.cu -- label remap, WTA, weight scaling and the TV/Huber refinement
// kernels.  Compiled with --fmad=false; every fused multiply-add is explicit
// so the results equal the CPU oracle bit for bit.
#include <cfloat>

#include <cuda_bf16.h>

#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

// remapsolution_kernel (stereo/stereo.cu:841-850)
__global__ void k_remap(float *__restrict__ out, const int32_t *__restrict__ lab, long n, float dmin,
                        float dstep)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __fadd_rn(__fmul_rn((float)lab[i], dstep), dmin);
}

// arg_min_kernel (stereo/stereo.cu:348-370)
__global__ void k_argmin(float *__restrict__ out, const float *__restrict__ vol, long npx, int D,
                         float dmin, float dstep)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx) return;
    const float *v = vol + i * D;
    float cm = FLT_MAX;
    int mi = 0;
    for (int z = 0; z < D; ++z)
        if (v[z] < cm) {
            cm = v[z];
            mi = z;
        }
    out[i] = __fadd_rn(dmin, __fmul_rn((float)mi, dstep));
}

// iu::math::mulC (stereo/stereo.cpp:136-137)
__global__ void k_scale(float *__restrict__ x, long n, float s)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = __fmul_rn(x[i], s);
}

__global__ void k_nchw_to_nhwc(const float *__restrict__ in, float *__restrict__ out, int C, long npx)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx * C) return;
    long p = i / C;
    int c = (int)(i - p * C);
    out[i] = in[(long)c * npx + p];
}

__global__ void k_bf16_to_f32(const __nv_bfloat16 *__restrict__ in, int cs, int C, long npx, float *__restrict__ out)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx * C) return;
    long p = i / C;
    int c = (int)(i - p * C);
    out[i] = __bfloat162float(in[p * cs + c]);
}

// warp_image_kernel on a point-sampled, clamp-addressed C4 texture
// (stereo/stereo.cu:830-839, 130-150): source column floor(x + 0.5 - u).
__global__ void k_warp(float4 *__restrict__ out, const float4 *__restrict__ in, const float *__restrict__ u,
                       int W, int H)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)W * H) return;
    int y = (int)(i / W), x = (int)(i - (long)y * W);
    float xf = __fsub_rn(__fadd_rn((float)x, 0.5f), u[i]);
    int sx = (int)floorf(xf);
    sx = sx < 0 ? 0 : (sx > W - 1 ? W - 1 : sx);
    out[i] = in[(long)y * W + sx];
}

// do_fitting_kernel, do_abs = false (stereo/stereo.cu:419-442)
__global__ void k_fit(const float *__restrict__ vol3, float2 *__restrict__ qf, long n, float step, float lam)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float c0 = vol3[i * 3], c1 = vol3[i * 3 + 1], c2 = vol3[i * 3 + 2];
    float hh = __fmul_rn(step, 0.25f);
    float a = __fmul_rn(__fdiv_rn(__fsub_rn(c0, c2), __fmul_rn(hh, 2.0f)), lam);
    float b = __fmul_rn(__fdiv_rn(__fsub_rn(__fadd_rn(c0, c2), __fmul_rn(2.0f, c1)), __fmul_rn(hh, hh)), lam);
    qf[i] = make_float2(a, fmaxf(0.0f, b));
}

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fmaxf(lo, fminf(v, hi)); }

// ttvqf_primal_kernel (stereo/stereo.cu:701-729); texture reads at x-1 / y-1
// are clamp-addressed, i.e. clamped indices.
__global__ void k_primal(float *__restrict__ u, float *__restrict__ u_, const float *__restrict__ u0,
                         const float2 *__restrict__ qf, const float2 *__restrict__ p,
                         const float2 *__restrict__ q, int W, int H, float tau, float half)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)W * H) return;
    int y = (int)(i / W), x = (int)(i - (long)y * W);
    long ixm = (long)y * W + (x > 0 ? x - 1 : 0);
    long iym = (long)(y > 0 ? y - 1 : 0) * W + x;
    float2 pc = p[i], qc = q[i];
    float Px = __fsub_rn(pc.x, qc.x), Py = __fsub_rn(pc.y, qc.y);
    float X = __fsub_rn(p[ixm].x, q[ixm].x);
    float Y = __fsub_rn(p[iym].y, q[iym].y);
    float div = __fsub_rn(__fadd_rn(__fsub_rn(Px, X), Py), Y);
    float un = __fmaf_rn(tau, div, u[i]);
    float2 ab = qf[i];
    float uz = u0[i];
    float inner = __fmaf_rn(-ab.y, uz, ab.x);
    float num = __fmaf_rn(-tau, inner, un);
    float den = __fmaf_rn(tau, ab.y, 1.0f);
    un = clampf(__fdiv_rn(num, den), __fsub_rn(uz, half), __fadd_rn(uz, half));
    u_[i] = __fsub_rn(__fmul_rn(2.0f, un), u_[i]);
    u[i] = un;
}

// prox_p with alpha = 0 (stereo/stereo.cu:752-757)
__device__ __forceinline__ float prox_p0(float v, float beta, float sigma, float w)
{
    if (fabsf(v) <= __fmul_rn(w, 0.0f)) return v;
    float m = fmaxf(0.0f, __fmaf_rn(-sigma, beta, fabsf(v)));
    float r = __fmul_rn(m, v > 0.0f ? 1.0f : -1.0f);
    return clampf(r, -w, w);
}

// thuberqf_dual_kernel (stereo/stereo.cu:773-796); Huber parameter eps was
// the constant 0.1 there.
__global__ void k_dual(float2 *__restrict__ p, float2 *__restrict__ q, const float *__restrict__ wx,
                       const float *__restrict__ wy, const float *__restrict__ u_, int W, int H,
                       float sigma, float C, float eps)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)W * H) return;
    int y = (int)(i / W), x = (int)(i - (long)y * W);
    float uc = u_[i];
    float dx = __fsub_rn(u_[(long)y * W + (x + 1 < W ? x + 1 : W - 1)], uc);
    float dy = __fsub_rn(u_[(long)(y + 1 < H ? y + 1 : H - 1) * W + x], uc);
    float2 pc = p[i], qc = q[i];
    float pnx = __fmaf_rn(sigma, dx, pc.x), pny = __fmaf_rn(sigma, dy, pc.y);
    float den = __fmaf_rn(sigma, eps, 1.0f);
    float wxx = wx[i], wyy = wy[i];
    p[i] = make_float2(clampf(__fdiv_rn(pnx, den), -wxx, wxx), clampf(__fdiv_rn(pny, den), -wyy, wyy));
    float qnx = __fmaf_rn(sigma, dx, qc.x), qny = __fmaf_rn(sigma, dy, qc.y);
    q[i] = make_float2(prox_p0(qnx, C, sigma, wxx), prox_p0(qny, C, sigma, wyy));
}

} // namespace

int remap(float *out, const int32_t *labels, long n, float dmin, float dstep, cudaStream_t st)
{
    {
        CNNCRF_PROF("remap", st);
        k_remap<<<ceil_div(n, 256), 256, 0, st>>>(out, labels, n, dmin, dstep);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int argmin(float *out, const float *vol, long npx, int D, float dmin, float dstep, cudaStream_t st)
{
    {
        CNNCRF_PROF("argmin", st);
        k_argmin<<<ceil_div(npx, 256), 256, 0, st>>>(out, vol, npx, D, dmin, dstep);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int scale(float *x, long n, float s, cudaStream_t st)
{
    {
        CNNCRF_PROF("scale", st);
        k_scale<<<ceil_div(n, 256), 256, 0, st>>>(x, n, s);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int nchw_to_nhwc(const float *in, float *out, int C, long npx, cudaStream_t st)
{
    {
        CNNCRF_PROF("nchw_to_nhwc", st);
        k_nchw_to_nhwc<<<ceil_div(npx * C, 256), 256, 0, st>>>(in, out, C, npx);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int bf16_to_f32(const void *in, int cs, int C, long npx, float *out, cudaStream_t st)
{
    {
        CNNCRF_PROF("bf16_to_f32", st);
        k_bf16_to_f32<<<ceil_div(npx * C, 256), 256, 0, st>>>((const __nv_bfloat16 *)in, cs, C, npx, out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int warp_rgba(float *out, const float *in, const float *u, int W, int H, cudaStream_t st)
{
    {
        CNNCRF_PROF("warp", st);
        k_warp<<<ceil_div((long)W * H, 256), 256, 0, st>>>((float4 *)out, (const float4 *)in, u, W, H);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int tv_fit(const float *vol3, float *qf, int W, int H, float step, float lam, cudaStream_t st)
{
    long n = (long)W * H;
    {
        CNNCRF_PROF("fit", st);
        k_fit<<<ceil_div(n, 256), 256, 0, st>>>(vol3, (float2 *)qf, n, step, lam);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

// cuda::fuseTHuberQuadFit's inner loop (stereo/stereo.cu:1141-1143,1159-1166):
// tau = sigma = 1/sqrt(8); per iteration u_ = u, primal, dual.
int tv_iterate(float *u, float *u_, const float *u0, const float *qf, float *p, float *q, const float *wx,
               const float *wy, int W, int H, float C, float eps, float step, int iters, cudaStream_t st)
{
    float L = (float)sqrt(8.0);
    float tau = 1.0f / L, sigma = 1.0f / L;
    float half = 0.5f * step;
    long n = (long)W * H;
    int nb = ceil_div(n, 256);
    for (int it = 0; it < iters; ++it) {
        CNNCRF_CUDA(cudaMemcpyAsync(u_, u, sizeof(float) * n, cudaMemcpyDeviceToDevice, st));
        {
            CNNCRF_PROF("primal", st);
            k_primal<<<nb, 256, 0, st>>>(u, u_, u0, (const float2 *)qf, (const float2 *)p, (const float2 *)q, W,
                                     H, tau, half);
        }
        {
            CNNCRF_PROF("dual", st);
            k_dual<<<nb, 256, 0, st>>>((float2 *)p, (float2 *)q, wx, wy, u_, W, H, sigma, C, eps);
        }
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
