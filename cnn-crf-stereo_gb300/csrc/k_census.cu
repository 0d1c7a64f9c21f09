// k_census.cu -- the non-CNN parts of the Stereo pipeline: grey images,
// census matching cost, image-gradient edge weights, the QuadDirect
// refinement and the left-right consistency check.
//
// Reference kernels: rgb_to_gray_kernel (stereo/stereo.cu:853-863),
// cost_vol_census_kernel (stereo/stereo.cu:306-346), calcEdgeImage =
// Gaussian(0.7) + filter_{x,y}_forward_kernel (stereo/stereo.cu:471-520,
// 1090-1095), do_fitting_kernel_volume + do_argmin_kernel_volume
// (stereo/stereo.cu:913-942, 1172-1194), leftrightcheck_kernel
// (stereo/stereo.cu:803-817).  The reference reads its images through CUDA
// textures; here every read is explicit index arithmetic:
//   clamp-addressed point reads at integer positions (the reference's texel
//   centres), and at fractional positions a linear interpolation in FP32
//   (t[i] + a * (t[i+1] - t[i]), a = position - floor(position)) where the
//   reference's texture unit interpolates with 8-bit weights.
// Compiled with --fmad=false: every result equals the CPU oracle bit for bit.
#include <cmath>

#include "../../include/cnncrf_fmath.h"
#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// linear read of row r at unnormalised texture coordinate u (texel centres at
// i + 0.5), clamp addressing
__device__ __forceinline__ float lerp_row(const float *__restrict__ r, int W, float u)
{
    const float t = __fsub_rn(u, 0.5f);
    const float f = floorf(t);
    const int i = (int)f;
    const float a = __fsub_rn(t, f);
    const float v0 = r[clampi(i, 0, W - 1)];
    if (a == 0.0f) return v0;
    const float v1 = r[clampi(i + 1, 0, W - 1)];
    return __fadd_rn(v0, __fmul_rn(a, __fsub_rn(v1, v0)));
}

__global__ void k_gray(const float *__restrict__ rgba, long n, float *__restrict__ gray)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float *px = rgba + 4 * i;
    gray[i] = (float)(0.2989 * (double)px[0] + 0.5870 * (double)px[1] + 0.1140 * (double)px[2]);
}

// one thread per pixel, all disparities; list[z] = the z-th disparity
__global__ void k_census(const float *__restrict__ g1, const float *__restrict__ g2, int W, int H, int fs,
                         const float *__restrict__ list, int D, float lambda, float *__restrict__ vol)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const float norm = (float)(fs * fs * 4);
    const float c1 = g1[(long)y * W + x];
    const float xx = __fadd_rn((float)x, 0.5f);
    for (int z = 0; z < D; ++z) {
        const float d = list[z];
        const float c2 = lerp_row(g2 + (long)y * W, W, __fsub_rn(xx, d));
        float cnt = 0.0f;
        for (int dy = -fs; dy <= fs; ++dy) {
            const int yy = clampi(y + dy, 0, H - 1);
            const float *r1 = g1 + (long)yy * W, *r2 = g2 + (long)yy * W;
            for (int dx = -fs; dx <= fs; ++dx) {
                if (dx == 0 && dy == 0) continue;
                const float i1 = r1[clampi(x + dx, 0, W - 1)];
                const float i2 = lerp_row(r2, W, __fsub_rn(__fadd_rn((float)(x + dx), 0.5f), d));
                if ((c1 > i1) != (c2 > i2)) cnt = __fadd_rn(cnt, 1.0f);
            }
        }
        vol[((long)y * W + x) * D + z] = __fmul_rn(lambda, __fdiv_rn(cnt, norm));
    }
}

// separable Gaussian, radius R, clamp-to-edge; horizontal then vertical pass
__global__ void k_gauss_h(const float *__restrict__ in, int W, int H, const float *__restrict__ w, int R,
                          float *__restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const float *r = in + (long)y * W;
    float s = 0.0f;
    for (int i = -R; i <= R; ++i) s = __fmaf_rn(w[i + R], r[clampi(x + i, 0, W - 1)], s);
    out[(long)y * W + x] = s;
}

__global__ void k_gauss_v(const float *__restrict__ in, int W, int H, const float *__restrict__ w, int R,
                          float *__restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    float s = 0.0f;
    for (int i = -R; i <= R; ++i) s = __fmaf_rn(w[i + R], in[(long)clampi(y + i, 0, H - 1) * W + x], s);
    out[(long)y * W + x] = s;
}

__device__ __forceinline__ float edge_weight(float diff, float alpha, float beta, float lambda)
{
    if (alpha > 0.0f)
        return fmaxf(__fmul_rn(lambda, cnncrf_expf(__fmul_rn(-alpha, cnncrf_powf(diff, beta)))), 1.0e-6f);
    return __fmul_rn(lambda, diff);
}

// forward differences of the smoothed image (the last column / row mirrors
// onto itself: difference 0)
__global__ void k_edges(const float *__restrict__ t, int W, int H, float alpha, float beta, float lambda,
                        float *__restrict__ wx, float *__restrict__ wy)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const long i = (long)y * W + x;
    const float c = t[i];
    const float dxv = fabsf(__fsub_rn(t[(long)y * W + min(x + 1, W - 1)], c));
    const float dyv = fabsf(__fsub_rn(t[(long)min(y + 1, H - 1) * W + x], c));
    wx[i] = edge_weight(dxv, alpha, beta, lambda);
    wy[i] = edge_weight(dyv, alpha, beta, lambda);
}

// parabola through the three costs around the solution's label
__global__ void k_quadfit_direct(float *__restrict__ u, const float *__restrict__ c1, long npx, int D, float dmin,
                                 float dstep)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx) return;
    const int z = (int)__fdiv_rn(__fsub_rn(u[i], dmin), dstep);
    if (z <= 0 || z >= D - 1) return; // no neighbour on one side: unchanged
    const float *c = c1 + i * D;
    const float a = __fdiv_rn(__fsub_rn(c[z - 1], c[z + 1]), __fmul_rn(dstep, 2.0f));
    const float b = fmaxf(1.0e-3f, __fdiv_rn(__fsub_rn(__fadd_rn(c[z - 1], c[z + 1]), __fmul_rn(2.0f, c[z])),
                                              __fmul_rn(dstep, dstep)));
    u[i] = __fadd_rn(u[i], __fdiv_rn(a, b));
}

__global__ void k_lr_check(const float *__restrict__ left, const float *__restrict__ right, int W, int H, float th,
                           float *__restrict__ out)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const long i = (long)y * W + x;
    const float d = left[i];
    const float dr = -lerp_row(right + (long)y * W, W, __fsub_rn(__fadd_rn((float)x, 0.5f), d));
    out[i] = fabsf(__fsub_rn(d, dr)) <= th ? d : -1.0f;
}

} // namespace

int rgb_to_gray(const float *rgba, long n, float *gray, cudaStream_t st)
{
    {
        CNNCRF_PROF("gray", st);
        k_gray<<<ceil_div(n, 256), 256, 0, st>>>(rgba, n, gray);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int census_volume(const float *g1, const float *g2, int W, int H, int fs, const float *d_list, int D, float lambda,
                  float *vol, cudaStream_t st)
{
    if (fs < 1 || fs > 16) return fail(CNNCRF_EINVAL, "census: filter size %d outside 1..16", fs);
    {
        CNNCRF_PROF("census", st);
        k_census<<<dim3(ceil_div(W, 128), H), 128, 0, st>>>(g1, g2, W, H, fs, d_list, D, lambda, vol);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

void gauss_weights(float sigma, int R, float *w)
{
    // exp(-i^2 / (2 sigma^2)) / sum, in double, rounded once (host; the CPU
    // oracle computes the same floats the same way)
    double s = 0.0, v[64];
    for (int i = -R; i <= R; ++i) s += (v[i + R] = std::exp(-(double)(i * i) / (2.0 * sigma * sigma)));
    for (int i = 0; i <= 2 * R; ++i) w[i] = (float)(v[i] / s);
}

int edge_weights(const float *gray, int W, int H, float alpha, float beta, float lambda, float *tmp, float *tmp2,
                 const float *d_gw, float *wx, float *wy, cudaStream_t st)
{
    const dim3 g(ceil_div(W, 128), H);
    {
        CNNCRF_PROF("gauss", st);
        k_gauss_h<<<g, 128, 0, st>>>(gray, W, H, d_gw, GAUSS_R, tmp);
        k_gauss_v<<<g, 128, 0, st>>>(tmp, W, H, d_gw, GAUSS_R, tmp2);
    }
    {
        CNNCRF_PROF("edges", st);
        k_edges<<<g, 128, 0, st>>>(tmp2, W, H, alpha, beta, lambda, wx, wy);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int quadfit_direct(float *u, const float *c1, long npx, int D, float dmin, float dstep, cudaStream_t st)
{
    {
        CNNCRF_PROF("quadfit", st);
        k_quadfit_direct<<<ceil_div(npx, 256), 256, 0, st>>>(u, c1, npx, D, dmin, dstep);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int lr_check(const float *left, const float *right, int W, int H, float th, float *out, cudaStream_t st)
{
    {
        CNNCRF_PROF("lr_check", st);
        k_lr_check<<<dim3(ceil_div(W, 128), H), 128, 0, st>>>(left, right, W, H, th, out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
