// k_misc.cu -- label remap, WTA, weight scaling, the refinement's warp and
// quadratic fit (the TV iterations are in k_tv.cu).  Compiled with --fmad=false; every fused multiply-add is explicit
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

} // namespace k
} // namespace cnncrf
