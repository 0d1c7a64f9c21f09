// k_conv_first_tc.cu -- the BF16 path's first convolution layers (feature net
// layer 1: 3x3, Cin = 1/3/5 -> 100; pairwise net layer 1: 3x3, 3 -> 64) on
// the tcgen05 tensor cores, replacing cudnnConvolutionForward + bias + tanh
// (stereo/operators/convolution.cpp:141-152, bias.cpp:58-67,
// activation.cpp:33-41) for the thin-input layers.
//
// K = kh * kw * Cin <= 64 is too thin for TMA-fed k-blocks: every thread
// instead gathers its own output pixel's patch (k = (ky, kx, ci) ascending,
// the FP32 path's order) from the normalised FP32 image, rounds it to BF16
// and writes it as one 128-byte row of the A tile in the 128-byte swizzle
// layout (16-byte chunk c of row r at chunk c ^ (r & 7)).  The weights are
// converted once per CTA into a resident B tile of the same layout.  A tile
// is 128 consecutive output pixels of one row: ceil(K / 16) UMMA K-steps
// (M = 128, N = NP) into the CTA's one 128-column TMEM accumulator, then the
// epilogue (tcgen05.ld, bias, tanh, BF16 NHWC output; each warp stages its 32
// pixels x 64 channels in shared memory and writes them by one TMA tensor store
// per box instead of 32 scattered pixel rows).  The steps of a tile
// run in order; four CTAs per SM (4 x 128 TMEM columns) hide each other's
// gather and store latency.  128 threads; every mbarrier wait is bounded and
// reports through the error flag.
#include <cstring>

#include <cuda_bf16.h>

#include "common.h"
#include "kernels.h"
#include "tc_util.cuh"

namespace cnncrf {
namespace k {

namespace {

constexpr int BM = 128;
constexpr int ROW = 128;           // bytes per swizzled row (64 bf16)
constexpr int A_BYTES = BM * ROW;  // 16 KB
constexpr int NUM_THREADS = 128;
constexpr uint32_t TMEM_COLS = 128; // one accumulator (N <= 128)
constexpr int CTAS_PER_SM = 4;      // 4 x 128 TMEM columns
constexpr int WT_LD = 128;         // row stride of the FP32 filter matrix [K][128]

struct FirstParams {
    const float *in;
    long in_pix, in_row, in_img;
    int Ho, Wo, Cin, kw, K, nk, n_img, tiles_x, num_tiles, cp_out;
    long out_img;
    const float *wt, *bias;
    __nv_bfloat16 *out;
    int *err;
    int ostage; // the output through shared memory and TMA stores (whole 64-channel boxes fit the row)
};
constexpr int OBUF = 32 * ROW; // a warp's output staging: 32 pixels x 64 BF16 channels

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *(uint32_t *)&h;
}

template <int NP>
__global__ void __launch_bounds__(NUM_THREADS)
    k_conv_first_tc(const __grid_constant__ CUtensorMap tmO, const FirstParams p)
{
    constexpr uint32_t IDESC = tc::idesc_bf16(BM, NP);
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint8_t *sA = smem;                   // [128 rows][128 B]
    uint8_t *sB = smem + A_BYTES;         // [NP rows][128 B]
    uint8_t *sO = sB + NP * ROW;          // [4 warps][OBUF] output staging (1024-byte aligned)
    float *sbias = (float *)(sO + 4 * OBUF);
    uint64_t *done = (uint64_t *)(sbias + NP); // [1]: the tile's MMAs
    uint32_t *tmem_slot = (uint32_t *)(done + 2);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    int *soff = (int *)(tmem_slot + 4); // [64]: patch element k's offset from the pixel's first input

    const int tid = threadIdx.x, warp = tid >> 5;
    const int nchunk = p.nk * 2; // 16-byte chunks of a row the MMAs read
    // resident weights: row n = output channel, chunk c = k in [8c, 8c + 8)
    for (int i = tid; i < NP * nchunk; i += NUM_THREADS) {
        const int n = i / nchunk, c = i - n * nchunk;
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int k0 = 8 * c + 2 * j;
            const float lo = k0 < p.K ? p.wt[(long)k0 * WT_LD + n] : 0.0f;
            const float hi = k0 + 1 < p.K ? p.wt[(long)(k0 + 1) * WT_LD + n] : 0.0f;
            w[j] = pack_bf16(lo, hi);
        }
        st_shared_v4(tc::smem_u32(sB + n * ROW + ((c ^ (n & 7)) << 4)), w[0], w[1], w[2], w[3]);
    }
    for (int i = tid; i < NP; i += NUM_THREADS) sbias[i] = p.bias ? p.bias[i] : 0.0f;
    // k = (ky, kx, ci) ascending -> ky * in_row + kx * in_pix + ci, once per CTA instead of per element
    for (int k = tid; k < p.K; k += NUM_THREADS) {
        const int tap = k / p.Cin, ci = k - tap * p.Cin;
        const int ky = tap / p.kw, kx = tap - ky * p.kw;
        soff[k] = (int)(ky * p.in_row + kx * p.in_pix) + ci;
    }
    if (tid == 0) {
        tc::mbar_init(&done[0], 1);
        *abort_flag = 0;
        tc::mbar_fence_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const int tiles_per_img = p.Ho * p.tiles_x;

    // epilogue of a finished tile: thread = pixel 32 * warp + lane (its TMEM lane)
    auto epilogue = [&](int t) {
        const int img = t / tiles_per_img, r = t - img * tiles_per_img;
        const int y = r / p.tiles_x, x = (r - y * p.tiles_x) * BM + tid;
        const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16);
        __nv_bfloat16 *o16 = p.out + img * p.out_img + ((long)y * p.Wo + x) * p.cp_out;
        float v[16];
        if (p.ostage) {
            const int xw = x - (tid & 31); // the warp's first pixel
            const tc::OStage os{&tmO, sO + warp * OBUF, xw < p.Wo, xw, y, img};
            const int lane = tid & 31;
            if (lane == 0) tc::bulk_wait_read0(); // the previous tile's last store has read the buffer
            __syncwarp();
#pragma unroll 1
            for (int c = 0; c < NP / 16; ++c) {
                tc::tmem_ld16(ta + c * 16, v); // warp-collective: every lane runs it
                uint32_t u[8];
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    u[j] = pack_bf16(tc::tanh_fast(v[2 * j] + sbias[c * 16 + 2 * j]),
                                     tc::tanh_fast(v[2 * j + 1] + sbias[c * 16 + 2 * j + 1]));
                tc::ostage_put<NP / 16>(os, lane, c, u); // (pixels past Wo are clipped by the store)
            }
            return;
        }
#pragma unroll 1
        for (int c = 0; c < NP / 16; ++c) {
            tc::tmem_ld16(ta + c * 16, v); // warp-collective: every lane runs it
            if (x < p.Wo) {
                uint32_t u[8];
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    u[j] = pack_bf16(tc::tanh_fast(v[2 * j] + sbias[c * 16 + 2 * j]),
                                     tc::tanh_fast(v[2 * j + 1] + sbias[c * 16 + 2 * j + 1]));
                uint4 *dst = (uint4 *)(o16 + c * 16);
                dst[0] = make_uint4(u[0], u[1], u[2], u[3]);
                dst[1] = make_uint4(u[4], u[5], u[6], u[7]);
            }
        }
    };

    int it = 0;
    bool ok = true;
    for (int t = blockIdx.x; t < p.num_tiles; t += gridDim.x, ++it) {
        // 1. this thread's A row: the patch of output pixel x0 + tid, BF16 (the previous tile's MMA,
        //    waited for below, has read the tile)
        {
            const int img = t / tiles_per_img, r = t - img * tiles_per_img;
            const int y = r / p.tiles_x, x = (r - y * p.tiles_x) * BM + tid;
            const float *src = p.in + img * p.in_img + (long)y * p.in_row + (long)x * p.in_pix;
            const uint32_t row = tc::smem_u32(sA + tid * ROW);
            for (int c = 0; c < nchunk; ++c) {
                uint32_t w[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    float f[2];
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int k = 8 * c + 2 * j + e;
                        f[e] = 0.0f;
                        if (k < p.K && x < p.Wo) f[e] = __ldg(src + soff[k]);
                    }
                    w[j] = pack_bf16(f[0], f[1]);
                }
                st_shared_v4(row + ((c ^ (tid & 7)) << 4), w[0], w[1], w[2], w[3]);
            }
        }
        // 2. the tensor core reads A through the async proxy; the previous epilogue's TMEM reads are done
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc::fence_before_sync();
        __syncthreads();
        // 3. MMAs of this tile
        if (tid == 0) {
            tc::fence_after_sync();
            const uint64_t da = tc::sdesc_sw128(tc::smem_u32(sA));
            const uint64_t db = tc::sdesc_sw128(tc::smem_u32(sB));
            for (int kk = 0; kk < p.nk; ++kk)
                tc::umma_bf16(tmem, da + 2 * kk, db + 2 * kk, IDESC, kk > 0 ? 1u : 0u);
            tc::umma_commit(&done[0]);
        }
        // 4. its epilogue; the outcome of the bounded wait is made uniform over the CTA
        const int got = tc::mbar_wait(&done[0], (uint32_t)it & 1u, abort_flag) ? 1 : 0;
        if (!__syncthreads_and(got)) {
            ok = false;
            break;
        }
        tc::fence_after_sync();
        epilogue(t);
        tc::fence_before_sync();
    }
    if (!ok && tid == 0) atomicExch(p.err, 1);
    if (p.ostage && (tid & 31) == 0) tc::bulk_wait0(); // the warp's stores are done before its buffer goes
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

template <int NP> size_t smem_bytes() { return 1024 + A_BYTES + NP * ROW + 4 * OBUF + NP * 4 + 2 * 8 + 16 + 64 * 4; }

template <int NP> int launch(FirstParams &p, cudaStream_t st)
{
    // the output as 4-D boxes of 64 channels x 32 pixels (whole boxes: cp_out >= 64 * ceil(NP / 64))
    CUtensorMap mo;
    std::memset(&mo, 0, sizeof mo);
    p.ostage = p.cp_out % 8 == 0 && p.cp_out >= 64 * ((NP + 63) / 64) && (p.out_img * 2) % 16 == 0 &&
               p.out_img >= (long)p.Ho * p.Wo * p.cp_out;
    if (p.ostage) {
        auto enc = tc::tensor_map_encoder();
        if (!enc) return fail(CNNCRF_ECUDA, "conv_first_tc: cuTensorMapEncodeTiled unavailable");
        cuuint64_t g[4] = {(cuuint64_t)p.cp_out, (cuuint64_t)p.Wo, (cuuint64_t)p.Ho, (cuuint64_t)p.n_img};
        cuuint64_t s[3] = {(cuuint64_t)p.cp_out * 2, (cuuint64_t)p.Wo * p.cp_out * 2, (cuuint64_t)p.out_img * 2};
        cuuint32_t b[4] = {64, 32, 1, 1}, e[4] = {1, 1, 1, 1};
        const CUresult r = enc(&mo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, p.out, g, s, b, e,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "conv_first_tc: output tensor map (%d)", (int)r);
    }
    int dev = 0, sms = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    // at most CTAS_PER_SM CTAs per SM (through shared memory): their accumulators fill the SM's 512 TMEM
    // columns, so no CTA waits in its allocation
    const size_t smem = std::max(smem_bytes<NP>(), (size_t)(200 * 1024 / CTAS_PER_SM));
    CNNCRF_CUDA(cudaFuncSetAttribute(k_conv_first_tc<NP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = std::min(p.num_tiles, CTAS_PER_SM * sms);
    {
        CNNCRF_PROF("conv_first_tc", st);
        k_conv_first_tc<NP><<<grid, NUM_THREADS, smem, st>>>(mo, p);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace

bool conv_first_tc_supported(const ConvArgs &a)
{
    const int K = a.kh * a.kw * a.Cin;
    return a.out16 && a.act == 1 && K >= 1 && K <= 64 && (a.Cout == 100 || a.Cout == 64) &&
           a.out_cs % 8 == 0 && a.out_cs >= (a.Cout == 100 ? 112 : 64);
}

int conv_first_tc(const ConvArgs &a, int *err, cudaStream_t st)
{
    if (!conv_first_tc_supported(a)) return fail(CNNCRF_EUNSUPPORTED, "conv_first_tc: layer not supported");
    if (((uintptr_t)a.out16 & 15) || !err) return fail(CNNCRF_EINVAL, "conv_first_tc: bad output");
    FirstParams p{};
    p.in = a.in, p.in_pix = a.in_pix, p.in_row = a.in_row, p.in_img = a.in_img;
    p.Ho = a.H - a.kh + 1, p.Wo = a.W - a.kw + 1;
    if (p.Ho < 1 || p.Wo < 1) return fail(CNNCRF_ESHAPE, "conv_first_tc: empty output");
    p.Cin = a.Cin, p.kw = a.kw, p.K = a.kh * a.kw * a.Cin, p.nk = ceil_div(p.K, 16);
    if ((long)(a.kh - 1) * a.in_row + (long)(a.kw - 1) * a.in_pix + a.Cin >= (1L << 31))
        return fail(CNNCRF_EUNSUPPORTED, "conv_first_tc: patch offsets beyond 32 bits");
    p.n_img = a.n_img, p.tiles_x = ceil_div(p.Wo, BM), p.num_tiles = a.n_img * p.Ho * p.tiles_x;
    p.cp_out = a.out_cs, p.out_img = a.out_img;
    p.wt = a.wt, p.bias = a.bias, p.out = (__nv_bfloat16 *)a.out16, p.err = err;
    return a.Cout == 100 ? launch<112>(p, st) : launch<64>(p, st);
}

} // namespace k
} // namespace cnncrf
