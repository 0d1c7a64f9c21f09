// k_conv_simt.cu -- the FP32 convolution of the bit-exact path.
//
// Implicit GEMM on the CUDA cores: out[p][co] = act(bias[co] + sum_k A[p][k] W[k][co])
// with p = output pixel, k = (ky, kx, ci) ci fastest.  Each output is
// accumulated in ascending k with one fmaf per term, so it equals the CPU
// oracle bit for bit (reference: cudnnConvolutionForward in
// CUDNN_CONVOLUTION mode + cudnnAddTensor + tanh, stereo/operators/
// convolution.cpp:141-152, bias.cpp:58-67, activation.cpp:33-41).
//
// Tiling: CTA = 128 pixels of one output row x 128 output channels, k-slices
// of 8 double-buffered in shared memory, 256 threads with 8x8 register tiles.
#include <cuda_bf16.h>

#include "../../include/cnncrf_fmath.h"
#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

constexpr int BM = 128, BN = 128, BK = 8, APAD = 4;

__device__ __forceinline__ float act_fn(float v, int act)
{
    if (act == 1) return cnncrf_tanhf(v);
    if (act == 2) return fabsf(v);
    if (act == 3) return fabsf(cnncrf_tanhf(v));
    return v;
}

__global__ void __launch_bounds__(256) k_conv_simt(ConvArgs a, int Ho, int Wo, int K)
{
    __shared__ __align__(16) float As[2][BK][BM + APAD];
    __shared__ __align__(16) float Bs[2][BK][BN];
    const int tid = threadIdx.x;
    const int oy = blockIdx.y;
    const int ox0 = blockIdx.x * BM;
    a.in += (long)blockIdx.z * a.in_img; // image of the batch
    if (a.out16) a.out16 = (char *)a.out16 + (long)blockIdx.z * a.out_img * 2;
    else a.out += (long)blockIdx.z * a.out_img;
    const int a_kk = tid & 7, a_p = tid >> 3;
    const int b_kk = tid >> 5, b_n = (tid & 31) * 4;
    const int tx = tid & 15, ty = tid >> 4;
    const int nsl = (K + BK - 1) / BK;

    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;

    float ra[4];
    float4 rb;
    auto loadA = [&](int s) {
        int kk = s * BK + a_kk;
        bool kv = kk < K;
        int ky = 0, kx = 0, ci = 0;
        if (kv) {
            int tap = kk / a.Cin;
            ci = kk - tap * a.Cin;
            ky = tap / a.kw;
            kx = tap - ky * a.kw;
        }
        const float *rowp = a.in + (long)(oy + ky) * a.in_row + (long)kx * a.in_pix + ci;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            int ox = ox0 + a_p + 32 * e;
            ra[e] = (kv && ox < Wo) ? __ldg(rowp + (long)ox * a.in_pix) : 0.0f;
        }
    };
    auto loadB = [&](int s) {
        int kk = s * BK + b_kk;
        rb = kk < K ? __ldg((const float4 *)(a.wt + (long)kk * BN + b_n)) : make_float4(0, 0, 0, 0);
    };
    auto storeAB = [&](int buf) {
#pragma unroll
        for (int e = 0; e < 4; ++e) As[buf][a_kk][a_p + 32 * e] = ra[e];
        *(float4 *)&Bs[buf][b_kk][b_n] = rb;
    };

    loadA(0);
    loadB(0);
    storeAB(0);
    __syncthreads();
    for (int s = 0; s < nsl; ++s) {
        const int cur = s & 1;
        if (s + 1 < nsl) {
            loadA(s + 1);
            loadB(s + 1);
        }
        const int kmax = min(BK, K - s * BK);
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            if (kk < kmax) {
                float4 a0 = *(const float4 *)&As[cur][kk][ty * 4];
                float4 a1 = *(const float4 *)&As[cur][kk][64 + ty * 4];
                float4 b0 = *(const float4 *)&Bs[cur][kk][tx * 4];
                float4 b1 = *(const float4 *)&Bs[cur][kk][64 + tx * 4];
                float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
                float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = __fmaf_rn(av[i], bv[j], acc[i][j]);
            }
        }
        if (s + 1 < nsl) storeAB(cur ^ 1);
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < 8; ++i) {
        int p = (i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4);
        int ox = ox0 + p;
        if (ox >= Wo) continue;
        float *dst = a.out16 ? nullptr : a.out + (long)oy * a.out_row + (long)ox * a.out_pix;
        __nv_bfloat16 *dst16 = a.out16 ? (__nv_bfloat16 *)a.out16 + ((long)oy * Wo + ox) * a.out_cs : nullptr;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int co = (j < 4) ? tx * 4 + j : 64 + tx * 4 + (j - 4);
            if (co < a.Cout) {
                float v = acc[i][j];
                if (a.bias) v = __fadd_rn(v, a.bias[co]);
                v = act_fn(v, a.act);
                if (dst16) dst16[co] = __float2bfloat16_rn(v);
                else dst[(long)co * a.out_ch] = v;
            }
        }
    }
}

// Packed FP32: two IEEE fmas, each rounded once (fma.rn.f32x2), on a pair of
// floats held in one 64-bit register -- the same values as two __fmaf_rn at
// half the instruction issue.
__device__ __forceinline__ unsigned long long pack2(float lo, float hi)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void fma2(unsigned long long &acc, unsigned long long a, unsigned long long b)
{
    asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(acc) : "l"(a), "l"(b));
}

// The same convolution with the channel tile cut to the layer's width (TN =
// 32, 64 or 112 output channels, for Cout <= TN) and the index arithmetic
// taken out of the k loop.  2 TN threads, each an 8 x 8 register tile (8
// pixels x 8 channels); k-slices of TK (7 at TN = 112, else 8), so that every
// thread loads one fixed k offset of each slice, for 128 TK / (2 TN) pixels
// whose offsets it computes once, and steps its (ky, kx, ci) from slice to
// slice without a division.  Per output the terms are accumulated in
// ascending k with one fmaf each, then + bias and the activation, as in
// k_conv_simt: the same bits.
template <int TN, int TK>
__global__ void __launch_bounds__(2 * TN, 2) k_conv_nt(ConvArgs a, int Ho, int Wo, int K)
{
    constexpr int NT = 2 * TN;      // threads
    constexpr int PA = BM * TK / NT; // pixels a thread loads per slice
    constexpr int PS = NT / TK;      // their stride
    constexpr int B4 = TK * TN / 4;  // float4 of a weight slice
    constexpr int BR = (B4 + NT - 1) / NT; // of them per thread
    static_assert(NT % TK == 0 && (BM * TK) % NT == 0, "k_conv_nt tile");
    __shared__ __align__(16) float As[2][TK][BM + APAD];
    __shared__ __align__(16) float Bs[2][TK][TN];
    const int tid = threadIdx.x;
    const int oy = blockIdx.y, ox0 = blockIdx.x * BM;
    a.in += (long)blockIdx.z * a.in_img; // image of the batch
    if (a.out16) a.out16 = (char *)a.out16 + (long)blockIdx.z * a.out_img * 2;
    else a.out += (long)blockIdx.z * a.out_img;
    const float *inb = a.in + (long)oy * a.in_row;
    // loader roles: k offset lk of every slice at pixels lp + PS j; weight float4s tid + NT r
    const int lk = tid % TK, lp = tid / TK;
    // compute roles: 16 pixel groups x TN / 8 channel groups, the pixel group
    // fastest, so that a quarter warp's 128-bit fragment loads read 128
    // contiguous bytes of the pixel row and the channel fragments are broadcasts
    const int ty = tid % 16, tx = tid / 16;
    long poff[PA];
    uint32_t pvalid = 0;
#pragma unroll
    for (int j = 0; j < PA; ++j) {
        const int ox = ox0 + lp + PS * j;
        poff[j] = (long)ox * a.in_pix;
        if (ox < Wo) pvalid |= 1u << j;
    }
    // (ky, kx, ci) of this thread's k in the current slice
    int kk = lk, ci = 0, kx = 0, ky = 0;
    if (kk < K) {
        const int tap = kk / a.Cin;
        ci = kk - tap * a.Cin;
        ky = tap / a.kw;
        kx = tap - ky * a.kw;
    }
    const int nfull = K / TK, nsl = (K + TK - 1) / TK;

    // accumulators of 8 pixels x 4 channel pairs (channels 2m, 2m+1 of the thread's 8)
    unsigned long long acc2[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int m = 0; m < 4; ++m) acc2[i][m] = 0ull;

    float ra[PA];
    float4 rb[BR];
    auto loadA = [&]() {
        const bool kv = kk < K;
        const float *src = inb + (long)ky * a.in_row + (long)kx * a.in_pix + ci;
#pragma unroll
        for (int j = 0; j < PA; ++j) ra[j] = (kv && (pvalid >> j & 1u)) ? __ldg(src + poff[j]) : 0.0f;
    };
    auto loadB = [&](int s) {
#pragma unroll
        for (int r = 0; r < BR; ++r) {
            const int f = tid + NT * r, k = s * TK + f / (TN / 4), n = (f % (TN / 4)) * 4;
            rb[r] = (f < B4 && k < K) ? __ldg((const float4 *)(a.wt + (long)k * BN + n)) : make_float4(0, 0, 0, 0);
        }
    };
    auto storeAB = [&](int buf) {
#pragma unroll
        for (int j = 0; j < PA; ++j) As[buf][lk][lp + PS * j] = ra[j];
#pragma unroll
        for (int r = 0; r < BR; ++r) {
            const int f = tid + NT * r;
            if (f < B4) *(float4 *)&Bs[buf][f / (TN / 4)][(f % (TN / 4)) * 4] = rb[r];
        }
    };
    auto advance = [&]() { // this thread's k of the next slice
        kk += TK;
        ci += TK;
        while (ci >= a.Cin) {
            ci -= a.Cin;
            if (++kx == a.kw) kx = 0, ++ky;
        }
    };
    auto step = [&](int cur, int k) {
        const float4 a0 = *(const float4 *)&As[cur][k][ty * 4];
        const float4 a1 = *(const float4 *)&As[cur][k][64 + ty * 4];
        const ulonglong2 b0 = *(const ulonglong2 *)&Bs[cur][k][tx * 4];
        const ulonglong2 b1 = *(const ulonglong2 *)&Bs[cur][k][TN / 2 + tx * 4];
        const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
        const unsigned long long bp[4] = {b0.x, b0.y, b1.x, b1.y};
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const unsigned long long ap = pack2(av[i], av[i]);
#pragma unroll
            for (int m = 0; m < 4; ++m) fma2(acc2[i][m], ap, bp[m]);
        }
    };

    loadA();
    loadB(0);
    storeAB(0);
    __syncthreads();
    for (int s = 0; s < nsl; ++s) {
        const int cur = s & 1;
        if (s + 1 < nsl) {
            advance();
            loadA();
            loadB(s + 1);
        }
        if (s < nfull) {
#pragma unroll
            for (int k = 0; k < TK; ++k) step(cur, k);
        } else {
            for (int k = 0; k < K - nfull * TK; ++k) step(cur, k);
        }
        if (s + 1 < nsl) storeAB(cur ^ 1);
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int ox = ox0 + ((i < 4) ? ty * 4 + i : 64 + ty * 4 + (i - 4));
        if (ox >= Wo) continue;
        float *dst = a.out16 ? nullptr : a.out + (long)oy * a.out_row + (long)ox * a.out_pix;
        __nv_bfloat16 *dst16 = a.out16 ? (__nv_bfloat16 *)a.out16 + ((long)oy * Wo + ox) * a.out_cs : nullptr;
        float accf[8];
#pragma unroll
        for (int m = 0; m < 4; ++m) asm("mov.b64 {%0, %1}, %2;" : "=f"(accf[2 * m]), "=f"(accf[2 * m + 1]) : "l"(acc2[i][m]));
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int co = (j < 4) ? tx * 4 + j : TN / 2 + tx * 4 + (j - 4);
            if (co < a.Cout) {
                float v = accf[j];
                if (a.bias) v = __fadd_rn(v, a.bias[co]);
                v = act_fn(v, a.act);
                if (dst16) dst16[co] = __float2bfloat16_rn(v);
                else dst[(long)co * a.out_ch] = v;
            }
        }
    }
}

// First layers (Cin <= 5): one thread per output pixel holds all COUT
// accumulators; its 3x3xCin patch sits in registers and the weights are read
// from shared memory as broadcast float4.  Same per-output order as above:
// k = (ky, kx, ci) ascending, one fmaf per term, then + bias, activation.
template <int COUT>
__global__ void __launch_bounds__(128) k_conv_first(ConvArgs a, int Ho, int Wo, int K)
{
    constexpr int CP = (COUT + 3) & ~3;
    extern __shared__ float4 wsm4[];
    float *wsm = (float *)wsm4; // [K][CP]
    for (int i = threadIdx.x; i < K * CP; i += blockDim.x) {
        int k = i / CP, co = i - k * CP;
        wsm[i] = a.wt[(long)k * BN + co];
    }
    __syncthreads();
    const int oy = blockIdx.y, ox = blockIdx.x * blockDim.x + threadIdx.x;
    if (ox >= Wo) return;
    a.in += (long)blockIdx.z * a.in_img; // image of the batch
    if (a.out16) a.out16 = (char *)a.out16 + (long)blockIdx.z * a.out_img * 2;
    else a.out += (long)blockIdx.z * a.out_img;
    // channel pairs (2m, 2m+1), one packed fma per pair and term
    unsigned long long acc2[CP / 2];
#pragma unroll
    for (int m = 0; m < CP / 2; ++m) acc2[m] = 0ull;
    for (int ky = 0; ky < a.kh; ++ky)
        for (int kx = 0; kx < a.kw; ++kx) {
            const float *src = a.in + (long)(oy + ky) * a.in_row + (long)(ox + kx) * a.in_pix;
            const int kb = (ky * a.kw + kx) * a.Cin;
            for (int ci = 0; ci < a.Cin; ++ci) {
                const float xv = __ldg(src + ci);
                const unsigned long long xp = pack2(xv, xv);
                const ulonglong2 *w = (const ulonglong2 *)(wsm + (kb + ci) * CP);
#pragma unroll
                for (int q = 0; q < CP / 4; ++q) {
                    const ulonglong2 wv = w[q];
                    fma2(acc2[2 * q], xp, wv.x);
                    fma2(acc2[2 * q + 1], xp, wv.y);
                }
            }
        }
    float acc[CP];
#pragma unroll
    for (int m = 0; m < CP / 2; ++m) asm("mov.b64 {%0, %1}, %2;" : "=f"(acc[2 * m]), "=f"(acc[2 * m + 1]) : "l"(acc2[m]));
#pragma unroll
    for (int co = 0; co < CP; ++co) {
        float v = acc[co];
        if (a.bias) v = __fadd_rn(v, a.bias[co]);
        acc[co] = act_fn(v, a.act);
    }
    const long pix = (long)oy * Wo + ox;
    if (a.out16) {
        __nv_bfloat16 *d16 = (__nv_bfloat16 *)a.out16 + pix * a.out_cs;
#pragma unroll
        for (int co = 0; co < COUT; co += 2) {
            const float v1 = co + 1 < COUT ? acc[co + 1] : 0.0f;
            *(__nv_bfloat162 *)(d16 + co) = __floats2bfloat162_rn(acc[co], v1);
        }
    } else {
        float *d = a.out + pix * a.Cout;
#pragma unroll
        for (int co = 0; co < COUT; ++co) d[co] = acc[co];
    }
}

__global__ void k_head2(const float *__restrict__ in, int npx, int Cin, const float *__restrict__ w,
                        float *__restrict__ out)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npx) return;
    in += (long)blockIdx.y * npx * Cin; // image of the batch
    out += (long)blockIdx.y * 2 * npx;
    const float *x = in + (long)p * Cin;
    float a0 = 0.0f, a1 = 0.0f;
    for (int ci = 0; ci < Cin; ++ci) {
        float v = x[ci];
        a0 = __fmaf_rn(w[ci], v, a0);
        a1 = __fmaf_rn(w[Cin + ci], v, a1);
    }
    out[p] = fabsf(a0);
    out[(long)npx + p] = fabsf(a1);
}

// Per pixel x / |x|, |x| = sqrt of the channel sum of squares in ascending c
// (one fmaf per term).  A CTA stages L2N pixels' channels in shared memory
// (row stride C + 1, odd: the per-pixel reads hit distinct banks) so the
// global reads and writes are contiguous, and one thread per pixel keeps the
// sequential sum.
constexpr int L2N = 64;
__global__ void __launch_bounds__(L2N) k_l2norm(float *__restrict__ f, long npx, int C)
{
    extern __shared__ float xs[]; // [L2N][C + 1]
    const long p0 = (long)blockIdx.x * L2N;
    const int n = (int)min((long)L2N, npx - p0), CS = C + 1;
    float *g = f + p0 * C;
    for (int i = threadIdx.x; i < n * C; i += L2N) {
        const int q = i / C;
        xs[q * CS + (i - q * C)] = g[i];
    }
    __syncthreads();
    if (threadIdx.x < n) {
        float *x = xs + threadIdx.x * CS;
        float s = 0.0f;
        for (int c = 0; c < C; ++c) s = __fmaf_rn(x[c], x[c], s);
        const float nr = __fsqrt_rn(s);
        for (int c = 0; c < C; ++c) x[c] = nr > 0.0f ? __fdiv_rn(x[c], nr) : 0.0f;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n * C; i += L2N) {
        const int q = i / C;
        g[i] = xs[q * CS + (i - q * C)];
    }
}

} // namespace

int conv_simt(const ConvArgs &args, cudaStream_t st)
{
    ConvArgs a = args;
    if (a.Cout > BN) return fail(CNNCRF_EINVAL, "conv_simt: Cout %d > %d", a.Cout, BN);
    int Ho = a.H - a.kh + 1, Wo = a.W - a.kw + 1;
    if (Ho <= 0 || Wo <= 0) return fail(CNNCRF_ESHAPE, "conv_simt: empty output");
    int K = a.kh * a.kw * a.Cin;
    const bool dense = a.out_pix == 0;
    if (dense) a.out_pix = a.Cout, a.out_row = (long)Wo * a.Cout, a.out_ch = 1;
    if (dense && K <= 45 && (a.Cout == 100 || a.Cout == 64) && a.Cout == (a.Cout & ~1)) {
        dim3 g(ceil_div(Wo, 128), Ho, a.n_img);
        size_t smem = sizeof(float) * (size_t)K * ((a.Cout + 3) & ~3);
        if (a.Cout == 100) {
            CNNCRF_PROF("conv_first", st);
            k_conv_first<100><<<g, 128, smem, st>>>(a, Ho, Wo, K);
        } else {
            CNNCRF_PROF("conv_first", st);
            k_conv_first<64><<<g, 128, smem, st>>>(a, Ho, Wo, K);
        }
        CNNCRF_CHECK_LAUNCH();
        return CNNCRF_OK;
    }
    dim3 grid(ceil_div(Wo, BM), Ho, a.n_img);
    {
        CNNCRF_PROF("conv_simt", st);
        if (a.Cout <= 32) k_conv_nt<32, 8><<<grid, 64, 0, st>>>(a, Ho, Wo, K);
        else if (a.Cout <= 64) k_conv_nt<64, 8><<<grid, 128, 0, st>>>(a, Ho, Wo, K);
        else if (a.Cout <= 112) k_conv_nt<112, 14><<<grid, 224, 0, st>>>(a, Ho, Wo, K);
        else k_conv_simt<<<grid, 256, 0, st>>>(a, Ho, Wo, K);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int conv_head2(const float *in, int npx, int Cin, const float *w, float *out, cudaStream_t st, int n_img)
{
    {
        CNNCRF_PROF("head2", st);
        k_head2<<<dim3(ceil_div(npx, 256), n_img), 256, 0, st>>>(in, npx, Cin, w, out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int l2norm(float *f, long npx, int C, cudaStream_t st)
{
    {
        CNNCRF_PROF("l2norm", st);
        const size_t sm = sizeof(float) * L2N * (size_t)(C + 1);
        if (sm > 48 * 1024) return fail(CNNCRF_EINVAL, "l2norm: %d channels", C);
        k_l2norm<<<ceil_div(npx, L2N), L2N, sm, st>>>(f, npx, C);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
