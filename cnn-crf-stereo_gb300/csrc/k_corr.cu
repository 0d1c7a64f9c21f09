// k_corr.cu -- FP32 correlation cost volume with the unary fused in.
//
// Restates kCorrelation_NHWC / kCorrelation_NHWC_interpolation
// (stereo/operators/stereocorrelation.cu:66-142, rectCorr = 0) followed by the
// channel softmax over D and the negation (stereo/operators/softmax.cpp:30-38,
// stereo/utils.cu:289-292), or by 1 - <fL,fR> for L2-normalised features.
// Compiled with --fmad=false; the dot products use explicit fmaf in channel
// order and the softmax sum follows the lane layout below, so the output is
// bit-identical to the CPU oracle.
//
// Block = one image row y, 32 pixels; the left tile and the band of right
// pixels those pixels can see are staged in shared memory (odd row stride:
// lanes read consecutive rows without bank conflicts).  One warp per pixel;
// lane j owns disparity indices k = j + 32 r.
#include <algorithm>
#include <cfloat>

#include <cuda_bf16.h>

#include "../../include/cnncrf_fmath.h"
#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

constexpr int PIX = 32;
constexpr int MAXP = 16; // D <= 512

__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

// TIN: feature element type (float: the bit-exact path; bf16: the tensor-core
// path's features); cs = channel stride of a pixel (>= C)
template <typename TIN>
__global__ void __launch_bounds__(256)
    k_corr(const TIN *__restrict__ fl, const TIN *__restrict__ fr, int H, int W, int C, int cs,
           const float *__restrict__ list, int D, int omin, int omax, int interp, int unary,
           float *__restrict__ out, long fps)
{
    extern __shared__ float sm[];
    fl += blockIdx.z * fps; // pair of the batch
    fr += blockIdx.z * fps;
    out += (long)blockIdx.z * H * W * D;
    const int y = blockIdx.y;
    const int x0 = blockIdx.x * PIX;
    const int CS = C + 1;
    const int xlo = max(0, x0 + omin);
    const int xhi = min(W - 1, x0 + PIX - 1 + omax);
    const int R = max(0, xhi - xlo + 1);
    const int npx = min(PIX, W - x0);
    float *sl = sm;                     // [PIX][CS]
    float *sr = sl + PIX * CS;          // [R][CS]
    float *sd = sr + (size_t)R * CS;    // [D]
    for (int i = threadIdx.x; i < npx * C; i += blockDim.x) {
        int p = i / C, c = i - p * C;
        sl[p * CS + c] = to_f(fl[((long)y * W + x0 + p) * cs + c]);
    }
    for (int i = threadIdx.x; i < R * C; i += blockDim.x) {
        int p = i / C, c = i - p * C;
        sr[p * CS + c] = to_f(fr[((long)y * W + xlo + p) * cs + c]);
    }
    for (int i = threadIdx.x; i < D; i += blockDim.x) sd[i] = list[i];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int P = (D + 31) >> 5;
    for (int pi = warp; pi < npx; pi += 8) {
        const int x = x0 + pi;
        const float *a = sl + pi * CS;
        float cv[MAXP];
#pragma unroll
        for (int r = 0; r < MAXP; ++r) {
            cv[r] = 0.0f;
            int kk = lane + 32 * r;
            if (r < P && kk < D) {
                float s = sd[kk];
                float w2 = (float)x + s;
                float acc = 0.0f;
                if (!interp) {
                    if (w2 >= 0.0f) {
                        int xs = x + (int)s;
                        if (xs <= W - 1) {
                            const float *b = sr + (xs - xlo) * CS;
                            for (int c = 0; c < C; ++c) acc = __fmaf_rn(a[c], b[c], acc);
                        }
                    }
                } else if (w2 >= 0.0f) {
                    int xa = (int)floorf(w2);
                    int xb = (int)(w2 + 1.0f);
                    float num = w2 - (float)xa;
                    float den = (float)xb - (float)xa;
                    // taps stay inside the staged band [xlo, xhi] (float rounding of
                    // w2 + 1 cannot step past it); xhi <= W - 1 also clamps the right edge
                    const float *b0 = sr + (min(max(xa, xlo), xhi) - xlo) * CS;
                    const float *b1 = sr + (min(max(xb, xlo), xhi) - xlo) * CS;
                    for (int c = 0; c < C; ++c) {
                        float y0 = b0[c], y1 = b1[c];
                        float it = y0 + ((y1 - y0) * num) / den;
                        acc = __fmaf_rn(a[c], it, acc);
                    }
                }
                cv[r] = acc;
            }
        }
        float *o = out + ((long)y * W + x) * D;
        if (unary == 0) {
            float m = -FLT_MAX;
#pragma unroll
            for (int r = 0; r < MAXP; ++r)
                if (r < P && lane + 32 * r < D) m = fmaxf(m, cv[r]);
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
            float s = 0.0f;
#pragma unroll
            for (int r = 0; r < MAXP; ++r) {
                if (r < P) {
                    int kk = lane + 32 * r;
                    float e = kk < D ? cnncrf_expf(cv[r] - m) : 0.0f;
                    cv[r] = e;
                    s = (r == 0) ? e : s + e;
                }
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, off);
#pragma unroll
            for (int r = 0; r < MAXP; ++r) {
                int kk = lane + 32 * r;
                if (r < P && kk < D) o[kk] = -(cv[r] / s);
            }
        } else {
#pragma unroll
            for (int r = 0; r < MAXP; ++r) {
                int kk = lane + 32 * r;
                if (r < P && kk < D) o[kk] = unary == 1 ? 1.0f - cv[r] : cv[r];
            }
        }
    }
}

// Integer disparities as a banded GEMM: for the 32 pixels x0.. of row y and
// every right pixel j of their band, T[p][j] = sum_c fL[c][p] * fR[c][j]
// (ascending c, one fmaf per term from 0: the same value as the per-pixel
// loop above), register-blocked 4 pixels x NJ band columns per thread; then
// one warp per pixel picks its D taps out of T and applies the unary.
constexpr int MAXNJ = 16;

template <typename TIN>
__global__ void __launch_bounds__(256)
    k_corr_band(const TIN *__restrict__ fl, const TIN *__restrict__ fr, int H, int W, int C, int cs,
                const float *__restrict__ list, int D, int omin, int omax, int NJ, int unary,
                float *__restrict__ out, long fps)
{
    extern __shared__ float sm[];
    fl += blockIdx.z * fps; // pair of the batch
    fr += blockIdx.z * fps;
    out += (long)blockIdx.z * H * W * D;
    const int y = blockIdx.y;
    const int x0 = blockIdx.x * PIX;
    const int RB = NJ * 32;                  // band columns computed (>= PIX + omax - omin)
    const int xlo = x0 + omin;               // band column 0 (may be < 0: zero filled)
    const int LS = PIX + 1, RS = RB + 1;     // odd row strides
    float *sl = sm;                          // [C][LS]
    float *sr = sl + (size_t)C * LS;         // [C][RS]
    float *sd = sr + (size_t)C * RS;         // [D]
    const int npx = min(PIX, W - x0);
    for (int i = threadIdx.x; i < PIX * C; i += blockDim.x) {
        int p = i / C, c = i - p * C;
        sl[c * LS + p] = p < npx ? to_f(fl[((long)y * W + x0 + p) * cs + c]) : 0.0f;
    }
    for (int i = threadIdx.x; i < RB * C; i += blockDim.x) {
        int j = i / C, c = i - j * C;
        int xr = xlo + j;
        sr[c * RS + j] = (xr >= 0 && xr < W) ? to_f(fr[((long)y * W + xr) * cs + c]) : 0.0f;
    }
    for (int i = threadIdx.x; i < D; i += blockDim.x) sd[i] = list[i];
    __syncthreads();

    const int tp = threadIdx.x & 7, tj = threadIdx.x >> 3;
    float acc[4][MAXNJ];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < MAXNJ; ++j) acc[i][j] = 0.0f;
    for (int c = 0; c < C; ++c) {
        const float *a = sl + c * LS + tp * 4;
        const float a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
        const float *b = sr + c * RS + tj * NJ;
#pragma unroll
        for (int j = 0; j < MAXNJ; ++j) {
            if (j < NJ) {
                const float bv = b[j];
                acc[0][j] = __fmaf_rn(a0, bv, acc[0][j]);
                acc[1][j] = __fmaf_rn(a1, bv, acc[1][j]);
                acc[2][j] = __fmaf_rn(a2, bv, acc[2][j]);
                acc[3][j] = __fmaf_rn(a3, bv, acc[3][j]);
            }
        }
    }
    __syncthreads(); // the tiles are dead: T reuses their storage
    float *T = sm;   // [PIX][RS]
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < MAXNJ; ++j)
            if (j < NJ) T[(tp * 4 + i) * RS + tj * NJ + j] = acc[i][j];
    float *sd2 = T + (size_t)PIX * RS;
    for (int i = threadIdx.x; i < D; i += blockDim.x) sd2[i] = list[i];
    __syncthreads();

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int P = (D + 31) >> 5;
    for (int pi = warp; pi < npx; pi += 8) {
        const int x = x0 + pi;
        float cv[MAXP];
#pragma unroll
        for (int r = 0; r < MAXP; ++r) {
            cv[r] = 0.0f;
            int kk = lane + 32 * r;
            if (r < P && kk < D) {
                float s = sd2[kk];
                float w2 = (float)x + s;
                if (w2 >= 0.0f) {
                    int xs = x + (int)s;
                    if (xs <= W - 1) cv[r] = T[pi * RS + (xs - xlo)];
                }
            }
        }
        float *o = out + ((long)y * W + x) * D;
        if (unary == 0) {
            float m = -FLT_MAX;
#pragma unroll
            for (int r = 0; r < MAXP; ++r)
                if (r < P && lane + 32 * r < D) m = fmaxf(m, cv[r]);
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, off));
            float sum = 0.0f;
#pragma unroll
            for (int r = 0; r < MAXP; ++r) {
                if (r < P) {
                    int kk = lane + 32 * r;
                    float e = kk < D ? cnncrf_expf(cv[r] - m) : 0.0f;
                    cv[r] = e;
                    sum = (r == 0) ? e : sum + e;
                }
            }
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) sum = sum + __shfl_xor_sync(0xffffffffu, sum, off);
#pragma unroll
            for (int r = 0; r < MAXP; ++r) {
                int kk = lane + 32 * r;
                if (r < P && kk < D) o[kk] = -(cv[r] / sum);
            }
        } else {
#pragma unroll
            for (int r = 0; r < MAXP; ++r) {
                int kk = lane + 32 * r;
                if (r < P && kk < D) o[kk] = unary == 1 ? 1.0f - cv[r] : cv[r];
            }
        }
    }
}

} // namespace

template <typename TIN>
static int corr_launch(const TIN *fl, const TIN *fr, int H, int W, int C, int cs, const float *d_list, int D,
                       int omin, int omax, bool interp, int unary, float *out, cudaStream_t st, int npairs,
                       long fps)
{
    if (D < 1 || D > 32 * MAXP) return fail(CNNCRF_EINVAL, "correlation: D=%d outside [1,%d]", D, 32 * MAXP);
    dim3 grid(ceil_div(W, PIX), H, npairs);
    const int NJ = ceil_div(PIX + omax - omin, 32);
    // phase 1 holds the two feature tiles, phase 2 the result tile T in the
    // same storage: allocate the larger of the two
    const size_t tiles = (size_t)C * (PIX + 1) + (size_t)C * (NJ * 32 + 1) + D;
    const size_t tres = (size_t)PIX * (NJ * 32 + 1) + D;
    const size_t band_smem = sizeof(float) * std::max(tiles, tres);
    if (!interp && NJ <= MAXNJ && band_smem <= 227 * 1024) {
        CNNCRF_CUDA(cudaFuncSetAttribute(k_corr_band<TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)band_smem));
        {
            CNNCRF_PROF("corr", st);
            k_corr_band<TIN><<<grid, 256, band_smem, st>>>(fl, fr, H, W, C, cs, d_list, D, omin, omax, NJ, unary, out,
                                                             fps);
        }
        CNNCRF_CHECK_LAUNCH();
        return CNNCRF_OK;
    }
    int R = PIX + omax - omin + 1;
    size_t smem = sizeof(float) * ((size_t)(PIX + R) * (C + 1) + D);
    if (smem > 227 * 1024)
        return fail(CNNCRF_EINVAL, "correlation: disparity band too wide (%zu bytes of shared memory)", smem);
    CNNCRF_CUDA(cudaFuncSetAttribute(k_corr<TIN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    {
        CNNCRF_PROF("corr", st);
        k_corr<TIN><<<grid, 256, smem, st>>>(fl, fr, H, W, C, cs, d_list, D, omin, omax, interp ? 1 : 0, unary, out,
                                              fps);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int correlation(const float *fl, const float *fr, int H, int W, int C, const float *d_list, int D, int omin,
                int omax, bool interp, int unary, float *out, cudaStream_t st, int npairs, long fps)
{
    return corr_launch<float>(fl, fr, H, W, C, C, d_list, D, omin, omax, interp, unary, out, st, npairs, fps);
}

int correlation_bf16(const void *fl, const void *fr, int H, int W, int C, int cs, const float *d_list, int D,
                     int omin, int omax, bool interp, int unary, float *out, cudaStream_t st, int npairs, long fps)
{
    return corr_launch<__nv_bfloat16>((const __nv_bfloat16 *)fl, (const __nv_bfloat16 *)fr, H, W, C, cs, d_list,
                                      D, omin, omax, interp, unary, out, st, npairs, fps);
}

} // namespace k
} // namespace cnncrf
