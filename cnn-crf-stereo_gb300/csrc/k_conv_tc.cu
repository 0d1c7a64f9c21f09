// k_conv_tc.cu -- BF16 implicit-GEMM convolution on the 5th-generation tensor
// cores (tcgen05), the BF16 path's replacement for cudnnConvolutionForward +
// cudnnAddTensor + tanh (stereo/operators/convolution.cpp:141-152,
// bias.cpp:58-67, activation.cpp:33-41).
//
// GEMM view: D[pixel][n] = sum_{tap, c} act[y+ky][x+kx][c] * W[n][tap][c]
// (kernel pre-flipped on the host: CUDNN_CONVOLUTION).  A tile is two M = 128
// halves of 128 output pixels that share every weight load; N = NP output
// channels; K runs over taps x 64-channel chunks of the NHWC input.  Paired
// tiles are 256 consecutive pixels of one row; where a row's width modulo 256
// lies in (0, 128] (the last paired tile would be mostly empty) the tiles are
// instead consecutive entries of the list of all rows' 128-pixel halves, so a
// tile's halves may come from two rows.
//
// Operand reuse: one shared-memory stage holds, for one kernel row ky and one
// 64-channel chunk, the 264-pixel window of input row y+ky that both halves
// read (a 128-row and a 136-row box, one after the other; with independent
// halves a 136-row window per half) and the weights of the kw taps of that row.  The kx taps read the same window
// shifted by kx pixels (a descriptor that starts kx 128-byte rows into the
// swizzled tile), so the input is loaded once per kernel row instead of once
// per tap.
//
// Persistent, warp-specialised CTA (224 threads, one per SM):
//   warp 0      TMA producer: per stage two 4-D boxes (64 ch x 128 / 136 px,
//               zero fill past the row end) and kw 2-D weight boxes (64 ch x NP),
//               128-byte swizzle
//   warps 1, 6  TMEM allocation (warp 1) and tcgen05.mma issue (M=128,
//               N=NP, K=16 steps), one thread per half / accumulator: two
//               issuers keep the tensor core fed with these short MMAs;
//               their commits free smem stages and hand finished tiles to
//               the epilogue
//   warp 7      mode 4 with ysm: TMA of the tile's layer-below activations
//               into a shared buffer (4 boxes of 64 channels x 128 pixels)
//               once the epilogue has released it, so the epilogue reads
//               them from shared memory instead of waiting on DRAM
//   warps 2..5  epilogue: tcgen05.ld of both halves (one pixel per thread
//               per half), bias + tanh, then store BF16 NHWC / L2-normalise
//               / apply the pairwise net's 1x1 head; or (mode 3, a training
//               step's input gradient) store the sums as FP32 NHWC; or (mode
//               4) multiply them by the layer below's tanh derivative
//               1 - y^2 and store them as FP32 NHWC and as the BF16 copy
//               with a zero border that the layer below's gradients read
// TMEM holds two tiles (four 128-column accumulators): the epilogue of tile i
// overlaps the MMAs of tile i+1.  Every mbarrier wait is bounded: on timeout
// the role raises the CTA abort flag and the global error flag, in-flight
// copies and MMAs are drained (again bounded) and TMEM is freed before exit.
#include <algorithm>
#include <array>
#include <atomic>
#include <iterator>
#include <map>
#include <mutex>
#include <vector>

#include <cuda.h>
#include <cuda_bf16.h>

#include "common.h"
#include "kernels.h"
#include "tc_util.cuh"

namespace cnncrf {
namespace k {

namespace {

constexpr int BM = 128;                 // pixels per half (UMMA M)
constexpr int TILE_PX = 2 * BM;         // pixels per paired tile
constexpr int HROWS = BM + 8;           // one half's input window: 128 px + up to 8 more for the kx taps
constexpr int AROWS = BM + HROWS;       // paired: 264 rows x 64 bf16 = 33 KB (loaded as 128 + 136 rows)
constexpr int NUM_THREADS = 384;
constexpr int Y_BOX = 64 * BM * 2;      // one 64-channel x 128-pixel box of the layer-below activations
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t ACC_STRIDE = 128;    // columns per accumulator (>= NP)
constexpr int MAX_STAGES = 4;
constexpr int OBUF = 32 * 128;          // an epilogue warp's output staging: 32 pixels x 64 BF16 channels

struct TcParams {
    int n_img, Hin, Win, Ho, Wo, kh, kw, cp_in, kchunks, kk_last, cout, cp_out, tiles_x, num_tiles, mode,
        stages, stage_bytes;
    int halves;      // 0: paired tiles; else the number of 128-pixel halves (tiles_x = halves per row)
    int a_bytes;     // the input window of a stage: AROWS or 2 * HROWS rows of 128 bytes
    const float *bias; // [NP], zero padded
    const float *head; // [2][NP] (mode 2)
    void *out;
    int *err;
    const __nv_bfloat16 *aux; // mode 4: y [n_img][Ho][Wo][aux_cs]
    __nv_bfloat16 *out16;     // mode 4: [n_img][Ho + 2 o16_ph][Wo + 2 o16_pw][o16_cs]
    int aux_cs, o16_cs, o16_ph, o16_pw;
    float *bias_part;         // mode 4 (optional): [gridDim.x * 8][cout] channel sums of the output
    int ysm, y_boxes;         // mode 4: aux through the shared buffer (y_boxes per half), else global loads
    int ostage;               // mode 0: the output through shared memory and TMA stores (64-channel boxes)
};

// Output pixel coordinates of half h of tile t; false if the half is past
// the end of the half list (the last tile of an odd count)
__device__ __forceinline__ bool half_coords(const TcParams &p, int t, int h, int &img, int &y, int &x0)
{
    if (p.halves == 0) {
        const int per = p.Ho * p.tiles_x;
        img = t / per;
        const int r = t - img * per;
        y = r / p.tiles_x;
        x0 = (r - y * p.tiles_x) * TILE_PX + h * BM;
        return true;
    }
    const int hi = 2 * t + h, hc = min(hi, p.halves - 1), per = p.Ho * p.tiles_x;
    img = hc / per;
    const int r = hc - img * per;
    y = r / p.tiles_x;
    x0 = (r - y * p.tiles_x) * BM;
    return hi < p.halves;
}

// Mode 4 epilogue of one half for this thread's pixel: dz of the layer below
// = the sums times 1 - y^2 as BF16 into the padded copy (and FP32 if p.out),
// plus the warp's per-channel sums into sacc.  All NP / 16 chunks unrolled;
// the caller loads y (load_dz_y) for both halves before either is used, so
// the tile waits on memory once.
template <int NP>
__device__ __forceinline__ void load_dz_y(const TcParams &p, bool valid, int img, int y, int x, uint4 (*yv)[2])
{
    const size_t pix = ((size_t)img * p.Ho + y) * p.Wo + x;
#pragma unroll
    for (int c = 0; c < NP / 16; ++c) {
        if (valid) {
            const uint4 *yp = (const uint4 *)(p.aux + pix * p.aux_cs + c * 16);
            yv[c][0] = yp[0], yv[c][1] = yp[1];
        } else {
            yv[c][0] = yv[c][1] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
}

// the same from the tile's shared buffer: half h's box b (channels 64 b .. 64 b + 63), pixel row r, in
// the 128-byte swizzle (16-byte chunk j of row r at chunk j ^ (r & 7))
template <int NP>
__device__ __forceinline__ void load_dz_y_smem(const uint8_t *ybuf, int y_boxes, int h, int r, uint4 (*yv)[2])
{
#pragma unroll
    for (int c = 0; c < NP / 16; ++c) {
        const uint8_t *row = ybuf + (h * y_boxes + c / 4) * Y_BOX + r * 128;
        const int j0 = 2 * (c % 4);
        yv[c][0] = *(const uint4 *)(row + ((j0 ^ (r & 7)) << 4));
        yv[c][1] = *(const uint4 *)(row + (((j0 + 1) ^ (r & 7)) << 4));
    }
}

// One half's chunk c of mode 4: the sums times 1 - y^2 into v (zero for an
// invalid pixel, so it adds nothing to the bias sums), stored as BF16 into the
// padded copy (and as FP32 if p.out).
template <int NP>
__device__ __forceinline__ void dz_chunk(const TcParams &p, uint32_t ta, int c, bool valid, size_t pix, size_t q16,
                                         const uint4 (&yc)[2], float (&v)[16], const tc::OStage *os)
{
    tc::tmem_ld16(ta + c * 16, v); // warp-collective
    const uint32_t yw[8] = {yc[0].x, yc[0].y, yc[0].z, yc[0].w, yc[1].x, yc[1].y, yc[1].z, yc[1].w};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const float a = __uint_as_float(yw[j] << 16), b = __uint_as_float(yw[j] & 0xffff0000u);
        v[2 * j] = valid ? v[2 * j] * (1.0f - a * a) : 0.0f;
        v[2 * j + 1] = valid ? v[2 * j + 1] * (1.0f - b * b) : 0.0f;
    }
    uint32_t u[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        u[j] = *(uint32_t *)&b2;
    }
    if (os) { // (warp-collective; an invalid pixel's zeros land in the border or past the tensor)
        tc::ostage_put<NP / 16>(*os, tc::lane_id(), c, u);
    } else if (valid) {
        uint4 *d16 = (uint4 *)(p.out16 + q16 * p.o16_cs + c * 16);
        d16[0] = make_uint4(u[0], u[1], u[2], u[3]);
        d16[1] = make_uint4(u[4], u[5], u[6], u[7]);
    }
    if (!valid) return;
    if (p.out) {
        float *o = (float *)p.out + pix * p.cp_out + c * 16;
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            if (c * 16 + 4 * g + 3 < p.cout)
                *(float4 *)(o + 4 * g) = make_float4(v[4 * g], v[4 * g + 1], v[4 * g + 2], v[4 * g + 3]);
            else
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (c * 16 + 4 * g + j < p.cout) o[4 * g + j] = v[4 * g + j];
        }
    }
}

// Mode 4 epilogue of one half's accumulator for this thread's pixel, chunk by
// chunk (all NP / 16 chunks unrolled; ya holds the pixel's layer-below
// activations), adding the warp's per-channel sums into wacc.
template <int NP>
__device__ __forceinline__ void epilogue_dz(const TcParams &p, uint32_t ta, bool valid, size_t pix, size_t q16,
                                            int lane, float *wacc, const uint4 (*ya)[2], const tc::OStage *os)
{
    constexpr int NC = NP / 16;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        float v[16];
        dz_chunk<NP>(p, ta, c, valid, pix, q16, ya[c], v, os);
        if (p.bias_part) {
            // the warp's 32 pixels summed per channel: each exchange halves the values a lane keeps;
            // lane L ends with channel c * 16 + (L >> 1), twice
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const bool up = lane & 16;
                const float keep = up ? v[i + 8] : v[i], give = up ? v[i] : v[i + 8];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, give, 16);
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const bool up = lane & 8;
                const float keep = up ? v[i + 4] : v[i], give = up ? v[i] : v[i + 4];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, give, 8);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const bool up = lane & 4;
                const float keep = up ? v[i + 2] : v[i], give = up ? v[i] : v[i + 2];
                v[i] = keep + __shfl_xor_sync(0xffffffffu, give, 4);
            }
            {
                const bool up = lane & 2;
                const float keep = up ? v[1] : v[0], give = up ? v[0] : v[1];
                v[0] = keep + __shfl_xor_sync(0xffffffffu, give, 2);
            }
            v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
            if (!(lane & 1)) wacc[c * 16 + (lane >> 1)] += v[0];
        }
    }
}

// 16 values times s as BF16 into 16-byte aligned dst (two 16-byte stores)
__device__ __forceinline__ void store_bf16_16(__nv_bfloat16 *dst, const float (&v)[16], float s)
{
    uint32_t u[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * j] * s, v[2 * j + 1] * s);
        u[j] = *(uint32_t *)&b2;
    }
    uint4 *d = (uint4 *)dst;
    d[0] = make_uint4(u[0], u[1], u[2], u[3]);
    d[1] = make_uint4(u[4], u[5], u[6], u[7]);
}

// One stage's MMAs of one half, fully unrolled: kw taps x nk K-steps.
// Descriptor arithmetic is in 16-byte units: +8 moves the A window one pixel
// row, +2 one 16-element K step, +NB*8 to the next tap's weight box (NB rows:
// NP, or NP / 2 per CTA of a pair, whose MMAs are M = 256 over both CTAs).
// `first` = 0 only for the tile's first stage (overwrite the accumulator).
template <int NP, bool PAIR, int KW, int NK>
__device__ __forceinline__ void issue_stage(uint32_t d, uint64_t a, uint64_t db, uint32_t first)
{
    constexpr int NB = PAIR ? NP / 2 : NP;
    constexpr uint32_t IDESC = tc::idesc_bf16(PAIR ? 2 * BM : BM, NP);
#pragma unroll
    for (int kx = 0; kx < KW; ++kx)
#pragma unroll
        for (int kk = 0; kk < NK; ++kk) {
            const uint32_t acc = (kx | kk) ? 1u : first;
            if constexpr (PAIR)
                tc::umma_bf16_pair(d, a + 8 * kx + 2 * kk, db + kx * (NB * 8) + 2 * kk, IDESC, acc);
            else
                tc::umma_bf16(d, a + 8 * kx + 2 * kk, db + kx * (NB * 8) + 2 * kk, IDESC, acc);
        }
}

template <int NP, bool PAIR, int KW>
__device__ __forceinline__ void issue_stage_nk(int nk, uint32_t d, uint64_t a, uint64_t db, uint32_t first)
{
    switch (nk) {
    case 1: issue_stage<NP, PAIR, KW, 1>(d, a, db, first); break;
    case 2: issue_stage<NP, PAIR, KW, 2>(d, a, db, first); break;
    case 3: issue_stage<NP, PAIR, KW, 3>(d, a, db, first); break;
    default: issue_stage<NP, PAIR, KW, 4>(d, a, db, first); break;
    }
}

// PAIR: launched as 2-CTA clusters.  Each CTA runs its own tile (the even CTA
// tile 2u, the odd one 2u + 1 of the pair's u-th step) with its own input
// window, but stages only half of each tap's weights (output channels NP/2 *
// rank ..); the even CTA issues M = 256 MMAs over both CTAs' operands, so a
// weight byte staged serves twice the pixels and the tensor core reads fewer
// shared-memory bytes per MMA FLOP.  Both CTAs' copies complete on the even
// CTA's full barriers, its MMA commits arrive on both CTAs' empty and tfull
// barriers, and both CTAs' epilogue warps release an accumulator on the even
// CTA's tempty barrier.
template <int NP, bool PAIR>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_conv_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmA2,
              const __grid_constant__ CUtensorMap tmB, const __grid_constant__ CUtensorMap tmY,
              const __grid_constant__ CUtensorMap tmO, const TcParams p)
{
    constexpr int NB = PAIR ? NP / 2 : NP; // weight rows (output channels) this CTA stages per tap
    constexpr int B_BYTES = NB * 128;      // one tap's 64-channel weight box
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = p.stages;
    const int STAGE = p.stage_bytes;
    uint8_t *ybuf = smem + S * STAGE; // mode 4 with ysm: [2 halves][y_boxes][Y_BOX]
    uint8_t *obuf = ybuf + (p.ysm ? 2 * p.y_boxes * Y_BOX : 0); // ostage: [8 epilogue warps][OBUF]
    uint64_t *full = (uint64_t *)(obuf + (p.ostage ? 8 * OBUF : 0));
    uint64_t *empty = full + S;
    uint64_t *tfull = empty + S;  // [buffer][half]
    uint64_t *tempty = tfull + 4; // [buffer][half]
    uint64_t *drain = tempty + 4; // one per issuer
    uint64_t *yfull = drain + 2, *yempty = yfull + 1;
    uint32_t *tmem_slot = (uint32_t *)(yempty + 1);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    volatile int *zero_flag = abort_flag + 1;
    float *sbias = (float *)(tmem_slot + 4);
    float *shead = sbias + NP;
    float *sacc = shead + 2 * NP; // mode 4 bias sums: [8 epilogue warps][NP]

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 2); // a commit from each issuer
        }
        for (int b = 0; b < 4; ++b) {
            tc::mbar_init(&tfull[b], 1);               // the half's issuer commits
            tc::mbar_init(&tempty[b], PAIR ? 8 : 4);   // one arrive per epilogue warp of the half (both CTAs)
        }
        tc::mbar_init(&drain[0], 1);
        tc::mbar_init(&drain[1], 1);
        tc::mbar_init(yfull, 1);
        tc::mbar_init(yempty, 8); // one arrive per epilogue warp
        *abort_flag = 0;
        *zero_flag = 0;
        tc::mbar_fence_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmA2);
        tc::prefetch_tmap(&tmB);
        if (p.ysm) tc::prefetch_tmap(&tmY);
        if (p.ostage) tc::prefetch_tmap(&tmO);
    }
    for (int i = threadIdx.x; i < NP; i += NUM_THREADS) sbias[i] = p.bias ? p.bias[i] : 0.0f;
    if (p.mode == 2)
        for (int i = threadIdx.x; i < 2 * NP; i += NUM_THREADS) shead[i] = p.head[i];
    if (p.bias_part)
        for (int i = threadIdx.x; i < 8 * NP; i += NUM_THREADS) sacc[i] = 0.0f;
    if (warp == 1) {
        if constexpr (PAIR) {
            tc::tmem_alloc_pair(tmem_slot, TMEM_COLS);
            tc::tmem_relinquish_pair();
        } else {
            tc::tmem_alloc(tmem_slot, TMEM_COLS);
            tc::tmem_relinquish();
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if constexpr (PAIR) tc::cluster_sync(); // the peer's barriers are initialised before any arrive on them
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const int kblocks = p.kh * p.kchunks; // stages per tile: (ky, chunk)
    // the tile loop: step u of this CTA (or pair) runs tile t = tile_of(u); a pair's odd CTA past the
    // end (odd tile count) repeats the last tile's loads and stores nothing
    const uint32_t rank = PAIR ? tc::cluster_ctarank() : 0u;
    const bool leader = rank == 0;
    const int u0 = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
    const int ustep = PAIR ? (int)(gridDim.x >> 1) : (int)gridDim.x;
    const int nsteps = PAIR ? (p.num_tiles + 1) / 2 : p.num_tiles;
    auto tile_of = [&](int u) { return PAIR ? 2 * u + (int)rank : u; };

    if (warp == 0) {
        if (lane == 0) {
            int stage = 0, issued = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int u = u0; u < nsteps && ok; u += ustep) {
                const int t = min(tile_of(u), p.num_tiles - 1);
                int img0, y0, x00, img1, y1, x01;
                half_coords(p, t, 0, img0, y0, x00);
                half_coords(p, t, 1, img1, y1, x01);
                for (int kb = 0; kb < kblocks; ++kb) {
                    const int ky = kb / p.kchunks, ch = kb - ky * p.kchunks;
                    if (!tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    uint8_t *sa = smem + stage * STAGE;
                    const int wc = (ky * p.kw) * p.cp_in + ch * 64; // the row's first tap, this chunk
                    if constexpr (PAIR) {
                        // both CTAs' bytes complete on the even CTA's barrier
                        const uint32_t fb = tc::mapa(tc::smem_u32(&full[stage]), 0);
                        if (leader) tc::mbar_expect_tx(&full[stage], 2 * STAGE);
                        if (p.halves == 0) {
                            tc::tma_load_4d_pair(sa, &tmA, fb, ch * 64, x00, y0 + ky, img0);
                            tc::tma_load_4d_pair(sa + BM * 128, &tmA2, fb, ch * 64, x01, y1 + ky, img1);
                        } else {
                            tc::tma_load_4d_pair(sa, &tmA2, fb, ch * 64, x00, y0 + ky, img0);
                            tc::tma_load_4d_pair(sa + HROWS * 128, &tmA2, fb, ch * 64, x01, y1 + ky, img1);
                        }
                        for (int kx = 0; kx < p.kw; ++kx)
                            tc::tma_load_2d_pair(sa + p.a_bytes + kx * B_BYTES, &tmB, fb, wc + kx * p.cp_in,
                                                 (int)rank * NB);
                    } else {
                        tc::mbar_expect_tx(&full[stage], STAGE);
                        if (p.halves == 0) {
                            // input pixels x0 .. x0 + 263 as rows 0 .. 263 (a 128-row and a 136-row box)
                            tc::tma_load_4d(sa, &tmA, &full[stage], ch * 64, x00, y0 + ky, img0);
                            tc::tma_load_4d(sa + BM * 128, &tmA2, &full[stage], ch * 64, x01, y1 + ky, img1);
                        } else { // a 136-row window per half
                            tc::tma_load_4d(sa, &tmA2, &full[stage], ch * 64, x00, y0 + ky, img0);
                            tc::tma_load_4d(sa + HROWS * 128, &tmA2, &full[stage], ch * 64, x01, y1 + ky, img1);
                        }
                        for (int kx = 0; kx < p.kw; ++kx)
                            tc::tma_load_2d(sa + p.a_bytes + kx * B_BYTES, &tmB, &full[stage], wc + kx * p.cp_in,
                                            0);
                    }
                    ++issued;
                    if (++stage == S) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
            }
            if (!ok && (!PAIR || leader)) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
                // let the copies already issued land before shared memory is released (a pair's full
                // barriers, which the odd CTA's copies complete on too, are the even CTA's)
                int st = stage;
                uint32_t ph = phase;
                for (int i = 0; i < S && i < issued; ++i) {
                    if (--st < 0) {
                        st = S - 1;
                        ph ^= 1;
                    }
                    tc::mbar_wait(&full[st], ph, zero_flag, 1u << 20);
                }
            } else if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
            }
        }
    } else if (warp == 7) {
        if (p.ysm && lane == 0) {
            // the tile's layer-below activations, once the epilogue has released the buffer
            int lt = 0, issued = 0;
            bool ok = true;
            for (int u = u0; u < nsteps; u += ustep, ++lt) {
                const int t = min(tile_of(u), p.num_tiles - 1);
                if (!tc::mbar_wait(yempty, ((uint32_t)lt & 1u) ^ 1u, abort_flag)) {
                    ok = false;
                    break;
                }
                tc::mbar_expect_tx(yfull, (uint32_t)(2 * p.y_boxes * Y_BOX));
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    int img, y, x0;
                    half_coords(p, t, h, img, y, x0); // a half past the list loads the last one's pixels
                    for (int b = 0; b < p.y_boxes; ++b)
                        tc::tma_load_4d(ybuf + (h * p.y_boxes + b) * Y_BOX, &tmY, yfull, b * 64, x0, y, img);
                }
                ++issued;
            }
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
                // the copies of the last issue land before shared memory is released
                if (issued) tc::mbar_wait(yfull, ((uint32_t)issued - 1u) & 1u, zero_flag, 1u << 20);
            }
        }
    } else if (warp == 1 || warp == 6) {
        // two MMA issuers, one per half: a single thread cannot issue this
        // tile's short MMAs as fast as the tensor core retires them
        if (lane == 0 && leader) {
            const int h = warp == 6 ? 1 : 0;
            int stage = 0, lt = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int u = u0; u < nsteps && ok; u += ustep, ++lt) {
                const int acc = 2 * (lt & 1) + h; // accumulator: TMEM buffer lt & 1, half h
                const uint32_t use = (uint32_t)lt >> 1;
                if (!tc::mbar_wait(&tempty[acc], (use & 1) ^ 1, abort_flag)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t d = tmem + acc * ACC_STRIDE;
                for (int kb = 0; kb < kblocks; ++kb) {
                    if (!tc::mbar_wait(&full[stage], phase, abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const int ch = kb % p.kchunks;
                    const int nk = (ch == p.kchunks - 1) ? p.kk_last : 4;
                    const uint32_t sa = tc::smem_u32(smem + stage * STAGE);
                    const uint64_t a = tc::sdesc_sw128(sa + h * (p.halves ? HROWS : BM) * 128);
                    const uint64_t db = tc::sdesc_sw128(sa + p.a_bytes);
                    const uint32_t first = kb == 0 ? 0u : 1u;
                    if (p.kw == 3) issue_stage_nk<NP, PAIR, 3>(nk, d, a, db, first);
                    else if (p.kw == 2) issue_stage_nk<NP, PAIR, 2>(nk, d, a, db, first);
                    else issue_stage_nk<NP, PAIR, 1>(nk, d, a, db, first);
                    if constexpr (PAIR) tc::umma_commit_pair(&empty[stage], 3);
                    else tc::umma_commit(&empty[stage]);
                    if (++stage == S) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (ok) {
                    if constexpr (PAIR) tc::umma_commit_pair(&tfull[acc], 3);
                    else tc::umma_commit(&tfull[acc]);
                }
            }
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
            }
            // every MMA of this thread completes before TMEM is released
            if constexpr (PAIR) tc::umma_commit_pair(&drain[h], 1);
            else tc::umma_commit(&drain[h]);
            tc::mbar_wait(&drain[h], 0, zero_flag, 1u << 22);
        }
    } else {
        // eight epilogue warps, two per SM sub-partition: warps 2..5 empty half 0's accumulator, warps 8..11
        // half 1's, each warp the TMEM lane quarter warp % 4 (one output pixel per thread)
        const int h = warp >= 8 ? 1 : 0;
        const int q = warp & 3;
        const int row = q * 32 + lane;
        float *wacc = sacc + (4 * h + q) * NP; // this warp's row of the mode 4 bias sums
        uint8_t *obw = obuf + (4 * h + q) * OBUF; // this warp's output staging (ostage)
        const uint32_t tempty_c = PAIR ? tc::mapa(tc::smem_u32(&tempty[0]), 0) : 0u;
        int lt = 0;
        for (int u = u0; u < nsteps; u += ustep, ++lt) {
            const bool tile_ok = tile_of(u) < p.num_tiles;
            const int t = min(tile_of(u), p.num_tiles - 1);
            const int acc = 2 * (lt & 1) + h; // accumulator: TMEM buffer lt & 1, half h
            const uint32_t use = (uint32_t)lt >> 1;
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&tfull[acc], use & 1, abort_flag) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
                break;
            }
            tc::fence_after_sync();
            // hand the accumulator back to its issuer (a pair's barriers are the even CTA's): one arrive
            // per warp once every lane's TMEM reads are done
            auto release = [&]() {
                tc::fence_before_sync();
                __syncwarp();
                if (lane == 0) {
                    if constexpr (PAIR) tc::mbar_arrive_cluster(tempty_c + 8u * (uint32_t)acc);
                    else tc::mbar_arrive(&tempty[acc]);
                }
            };
            int img, y, x0;
            const bool hok = half_coords(p, t, h, img, y, x0) && tile_ok;
            const int x = x0 + row;
            const bool valid = hok && x < p.Wo;
            const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + acc * ACC_STRIDE;
            const size_t pix = ((size_t)img * p.Ho + y) * p.Wo + x;
            if (p.mode == 4) {
                uint4 ya[NP / 16][2];
                if (p.ysm) {
                    int got = 1;
                    if (lane == 0) got = tc::mbar_wait(yfull, (uint32_t)lt & 1u, abort_flag) ? 1 : 0;
                    got = __shfl_sync(0xffffffffu, got, 0);
                    if (!got) {
                        *abort_flag = 1;
                        atomicExch(p.err, 1);
                        break;
                    }
                    load_dz_y_smem<NP>(ybuf, p.y_boxes, h, row, ya);
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(yempty); // the buffer may take the next tile's activations
                } else {
                    load_dz_y<NP>(p, valid, img, y, x, ya);
                }
                const size_t q16 =
                    ((size_t)img * (p.Ho + 2 * p.o16_ph) + y + p.o16_ph) * (p.Wo + 2 * p.o16_pw) + x + p.o16_pw;
                // the padded copy through the staging buffer: boxes at (x + o16_pw, y + o16_ph) of the padded
                // tensor (a pixel past Wo holds zeros, which is what the border holds)
                const tc::OStage os{&tmO, obw, hok && x0 + q * 32 < p.Wo, x0 + q * 32 + p.o16_pw, y + p.o16_ph, img};
                if (p.ostage) {
                    if (lane == 0) tc::bulk_wait_read0();
                    __syncwarp();
                }
                epilogue_dz<NP>(p, ta, valid, pix, q16, lane, wacc, ya, p.ostage ? &os : nullptr);
                release();
                continue;
            }
            // the TMEM reads are warp-collective: every lane runs them
            float v[16];
            float sc = 1.0f;
            if (p.mode == 1) { // pass 1: squared norm of tanh(acc + bias)
                float s2 = 0.0f;
#pragma unroll 1
                for (int c = 0; c < NP / 16; ++c) {
                    tc::tmem_ld16(ta + c * 16, v);
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const float f = tc::tanh_fast(v[j] + sbias[c * 16 + j]);
                        s2 = fmaf(f, f, s2);
                    }
                }
                sc = s2 > 0.0f ? rsqrtf(s2) : 0.0f;
            }
            __nv_bfloat16 *o16 = (__nv_bfloat16 *)p.out + pix * p.cp_out;
            // mode 0 through shared memory: the warp's 32 pixels x 64 channels per TMA store, in the 128-byte
            // swizzle (16-byte unit j of pixel row r at unit j ^ (r & 7)), so every store is a whole box
            const bool tstore = p.ostage && (p.mode == 0 || p.mode == 1);
            const tc::OStage os{&tmO, obw, hok && x0 + q * 32 < p.Wo, x0 + q * 32, y, img};
            if (tstore) { // the previous tile's last store has read the buffer
                if (lane == 0) tc::bulk_wait_read0();
                __syncwarp();
            }
            float a0 = 0.0f, a1 = 0.0f;
#pragma unroll 1
            for (int c = 0; c < NP / 16; ++c) {
                tc::tmem_ld16(ta + c * 16, v);
                if (c == NP / 16 - 1) release(); // the accumulator's last read
                if (p.mode == 3) {
                    if (valid) {
                        float *o = (float *)p.out + pix * p.cp_out + c * 16;
#pragma unroll
                        for (int g = 0; g < 4; ++g) {
                            if (c * 16 + 4 * g + 3 < p.cout)
                                *(float4 *)(o + 4 * g) = make_float4(v[4 * g], v[4 * g + 1], v[4 * g + 2],
                                                                     v[4 * g + 3]);
                            else
#pragma unroll
                                for (int j = 0; j < 4; ++j)
                                    if (c * 16 + 4 * g + j < p.cout) o[4 * g + j] = v[4 * g + j];
                        }
                    }
                    continue;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = tc::tanh_fast(v[j] + sbias[c * 16 + j]);
                if (p.mode == 2) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        a0 = fmaf(v[j], shead[c * 16 + j], a0);
                        a1 = fmaf(v[j], shead[NP + c * 16 + j], a1);
                    }
                    if (p.out16 && valid) // the tanh outputs too (a training step's backward reads them)
                        store_bf16_16(p.out16 + pix * p.o16_cs + c * 16, v, 1.0f);
                } else if (tstore) {
                    uint32_t u[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * j] * sc, v[2 * j + 1] * sc);
                        u[j] = *(uint32_t *)&b2;
                    }
                    tc::ostage_put<NP / 16>(os, lane, c, u);
                    if (p.mode == 1 && p.out16 && valid) // the features before the normalisation too
                        store_bf16_16(p.out16 + pix * p.o16_cs + c * 16, v, 1.0f);
                } else if (valid) {
                    store_bf16_16(o16 + c * 16, v, sc);
                    if (p.mode == 1 && p.out16) // the features before the normalisation too
                        store_bf16_16(p.out16 + pix * p.o16_cs + c * 16, v, 1.0f);
                }
            }
            if (p.mode == 2 && valid) { // [img][2][Ho][Wo]
                const size_t plane = (size_t)p.Ho * p.Wo;
                float *o = (float *)p.out + (size_t)img * 2 * plane;
                o[(size_t)y * p.Wo + x] = fabsf(a0);
                o[plane + (size_t)y * p.Wo + x] = fabsf(a1);
            }
        }
        if (p.ostage && lane == 0) tc::bulk_wait0(); // the warp's stores are done before its buffer goes
    }
    __syncthreads();
    if (p.bias_part) // this CTA's eight partial sums per channel (one per epilogue warp)
        for (int i = threadIdx.x; i < 8 * p.cout; i += NUM_THREADS)
            p.bias_part[((size_t)blockIdx.x * 8 + i / p.cout) * p.cout + i % p.cout] =
                sacc[(i / p.cout) * NP + i % p.cout];
    if constexpr (PAIR) tc::cluster_sync(); // neither CTA leaves while the other may use its memory
    if (warp == 1) {
        tc::fence_after_sync();
        if constexpr (PAIR) tc::tmem_dealloc_pair(tmem, TMEM_COLS);
        else tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// NB: the weight rows a CTA stages per tap (NP, or NP / 2 in a pair)
inline int stage_bytes(int a_bytes, int kw, int NB) { return a_bytes + kw * NB * 128; }

inline size_t smem_bytes(int NP, int NB, int stages, int a_bytes, int kw, int mode, int ybytes = 0)
{
    return 1024 + (size_t)stages * stage_bytes(a_bytes, kw, NB) + ybytes + (2 * stages + 12) * 8 + 16 +
           (mode == 4 ? 11 : (mode == 2 ? 3 : 1)) * NP * 4;
}

std::atomic<int> g_pairs{1}; // CTA pairs (cta_group::2) where the device can co-schedule them

// the conv tuning table: layer shape -> fastest form (conv_tc_autotune)
struct ConvTuned {
    ConvForm form;
    float ms;
};
std::mutex g_tune_mu;
std::map<std::array<int, CONV_KEY>, ConvTuned> g_tune;

std::array<int, CONV_KEY> conv_key(const TcConvArgs &a)
{
    return {a.n_img, a.Hin, a.Win, a.cp_in, a.cin, a.np, a.cout, a.kh, a.kw, a.mode};
}

bool conv_form_lookup(const TcConvArgs &a, ConvForm *f)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(conv_key(a));
    if (it == g_tune.end()) return false;
    *f = it->second.form;
    return true;
}

// Co-resident 2-CTA clusters of k_conv_tc<NP, true> at `smem` bytes per CTA (0: none), cached per size.
template <int NP> int pair_clusters(size_t smem)
{
    static std::mutex mu;
    static std::map<size_t, int> cache;
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(smem);
    if (it != cache.end()) return it->second;
    int n = 0;
    if (cudaFuncSetAttribute(k_conv_tc<NP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) ==
        cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 2, at[0].val.clusterDim.y = 1, at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(2, 1, 1), cfg.blockDim = dim3(NUM_THREADS, 1, 1), cfg.dynamicSmemBytes = smem;
        cfg.attrs = at, cfg.numAttrs = 1;
        if (cudaOccupancyMaxActiveClusters(&n, (void *)k_conv_tc<NP, true>, &cfg) != cudaSuccess) n = 0;
    }
    cudaGetLastError(); // a refused query leaves no sticky error: the single-CTA kernel runs instead
    cache[smem] = n;
    return n;
}

template <int NP> int launch(const TcConvArgs &a, TcParams &p, cudaStream_t st)
{
    auto enc = tc::tensor_map_encoder();
    if (!enc) return fail(CNNCRF_ECUDA, "conv_tc: cuTensorMapEncodeTiled unavailable");
    CUtensorMap ma, mb;
    cuuint64_t gA[4] = {(cuuint64_t)a.cp_in, (cuuint64_t)a.Win, (cuuint64_t)a.Hin, (cuuint64_t)a.n_img};
    cuuint64_t sA[3] = {(cuuint64_t)a.cp_in * 2, (cuuint64_t)a.Win * a.cp_in * 2,
                        (cuuint64_t)a.Hin * a.Win * a.cp_in * 2};
    cuuint32_t bA[4] = {64, BM, 1, 1}, bA2[4] = {64, AROWS - BM, 1, 1};
    cuuint32_t eA[4] = {1, 1, 1, 1};
    CUtensorMap ma2;
    CUresult r = enc(&ma, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)a.in, gA, sA, bA, eA,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "conv_tc: activation tensor map (%d)", (int)r);
    r = enc(&ma2, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)a.in, gA, sA, bA2, eA, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "conv_tc: activation tensor map (%d)", (int)r);
    int dev = 0, sms = 0, maxsm = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // Shared-memory plan for nb weight rows per tap: mode 4's layer-below activations through a shared
    // buffer when it fits beside two stages (their global loads stalled the epilogue more than a third stage
    // gains), then the output staging for TMA stores if it fits too, then as many stages as fit.
    p.y_boxes = (NP + 63) / 64;
    const int ybytes = 2 * p.y_boxes * Y_BOX;
    // modes 0 and 1: the BF16 output (out, cp_out channels); mode 4: its padded BF16 copy (out16)
    const bool m4 = a.mode == 4;
    const int ocs = m4 ? a.o16_cs : a.cp_out, opw = m4 ? a.o16_pw : 0, oph = m4 ? a.o16_ph : 0;
    const bool ost_ok = (a.mode == 0 || a.mode == 1 || m4) && ocs % 8 == 0 && ocs >= 64 * ((NP + 63) / 64);
    // the form: the caller's, else the tuned one for this shape, else the defaults
    ConvForm form = a.form;
    if (form.pair < 0 && form.stages == 0) conv_form_lookup(a, &form);
    const int smax = form.stages >= 2 ? std::min(form.stages, MAX_STAGES) : MAX_STAGES;
    auto plan = [&](int nb, int &ysm, int &ost, int &stages) -> size_t {
        ysm = m4 && smem_bytes(NP, nb, 2, p.a_bytes, a.kw, a.mode, ybytes) <= (size_t)maxsm ? 1 : 0;
        const int yb = ysm ? ybytes : 0;
        ost = ost_ok && smem_bytes(NP, nb, 2, p.a_bytes, a.kw, a.mode, yb + 8 * OBUF) <= (size_t)maxsm ? 1 : 0;
        const int extra = yb + (ost ? 8 * OBUF : 0);
        stages = 0;
        for (int s = smax; s >= 2 && !stages; --s)
            if (smem_bytes(NP, nb, s, p.a_bytes, a.kw, a.mode, extra) <= (size_t)maxsm) stages = s;
        return smem_bytes(NP, nb, std::max(stages, 2), p.a_bytes, a.kw, a.mode, extra);
    };
    // CTA pairs when there are two tiles to pair and the device co-schedules the clusters
    bool pair = (form.pair < 0 ? g_pairs.load() != 0 : form.pair != 0) && p.num_tiles >= 2;
    int nclusters = 0;
    if (pair) {
        int ysm, ost, stages;
        const size_t sm = plan(NP / 2, ysm, ost, stages);
        nclusters = stages ? pair_clusters<NP>(sm) : 0;
        pair = nclusters > 0;
    }
    const int NB = pair ? NP / 2 : NP;
    const size_t smem = plan(NB, p.ysm, p.ostage, p.stages);
    p.stage_bytes = stage_bytes(p.a_bytes, a.kw, NB);
    if (!p.stages) return fail(CNNCRF_EUNSUPPORTED, "conv_tc: two stages of %d bytes exceed shared memory", p.stage_bytes);
    const int taps = a.kh * a.kw;
    cuuint64_t gB[2] = {(cuuint64_t)taps * a.cp_in, (cuuint64_t)NP};
    cuuint64_t sB[1] = {(cuuint64_t)taps * a.cp_in * 2};
    cuuint32_t bB[2] = {64, (cuuint32_t)NB};
    cuuint32_t eB[2] = {1, 1};
    r = enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)a.wt, gB, sB, bB, eB, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "conv_tc: weight tensor map (%d)", (int)r);
    CUtensorMap my = ma; // unused unless ysm
    if (p.ysm) {
        cuuint64_t gY[4] = {(cuuint64_t)a.aux_cs, (cuuint64_t)p.Wo, (cuuint64_t)p.Ho, (cuuint64_t)a.n_img};
        cuuint64_t sY[3] = {(cuuint64_t)a.aux_cs * 2, (cuuint64_t)p.Wo * a.aux_cs * 2,
                            (cuuint64_t)p.Ho * p.Wo * a.aux_cs * 2};
        cuuint32_t bY[4] = {64, BM, 1, 1}, eY[4] = {1, 1, 1, 1};
        r = enc(&my, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)a.aux, gY, sY, bY, eY, CU_TENSOR_MAP_INTERLEAVE_NONE,
                CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "conv_tc: activation (mode 4) tensor map (%d)", (int)r);
    }
    CUtensorMap mo = ma; // unused unless ostage
    if (p.ostage) {
        const cuuint64_t ow = (cuuint64_t)p.Wo + 2 * opw, oh = (cuuint64_t)p.Ho + 2 * oph;
        cuuint64_t gO[4] = {(cuuint64_t)ocs, ow, oh, (cuuint64_t)a.n_img};
        cuuint64_t sO[3] = {(cuuint64_t)ocs * 2, ow * ocs * 2, oh * ow * ocs * 2};
        cuuint32_t bO[4] = {64, 32, 1, 1}, eO[4] = {1, 1, 1, 1};
        r = enc(&mo, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, m4 ? a.out16 : a.out, gO, sO, bO, eO,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "conv_tc: output tensor map (%d)", (int)r);
    }
    if (pair) {
        // one cluster per pair of co-resident SMs, each running tile pairs until the list ends
        const int grid = 2 * std::min(nclusters, (p.num_tiles + 1) / 2);
        if (a.bias_splits) *a.bias_splits = 8 * grid;
        CNNCRF_CUDA(cudaFuncSetAttribute(k_conv_tc<NP, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 2, at[0].val.clusterDim.y = 1, at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(grid, 1, 1), cfg.blockDim = dim3(NUM_THREADS, 1, 1), cfg.dynamicSmemBytes = smem;
        cfg.stream = st, cfg.attrs = at, cfg.numAttrs = 1;
        {
            CNNCRF_PROF("conv_tc", st);
            CNNCRF_CUDA(cudaLaunchKernelEx(&cfg, k_conv_tc<NP, true>, ma, ma2, mb, my, mo, (const TcParams)p));
        }
    } else {
        const int grid = std::min(p.num_tiles, sms);
        if (a.bias_splits) *a.bias_splits = 8 * grid;
        CNNCRF_CUDA(cudaFuncSetAttribute(k_conv_tc<NP, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        {
            CNNCRF_PROF("conv_tc", st);
            k_conv_tc<NP, false><<<grid, NUM_THREADS, smem, st>>>(ma, ma2, mb, my, mo, p);
        }
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace

void conv_tc_set_pairs(bool on) { g_pairs.store(on ? 1 : 0); }
bool conv_tc_pairs() { return g_pairs.load() != 0; }

int conv_forms_count()
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    return (int)g_tune.size();
}

bool conv_form_entry(int i, int key[CONV_KEY], ConvForm *f, float *ms)
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    if (i < 0 || i >= (int)g_tune.size()) return false;
    auto it = g_tune.begin();
    std::advance(it, i);
    for (int j = 0; j < CONV_KEY; ++j) key[j] = it->first[j];
    *f = it->second.form;
    *ms = it->second.ms;
    return true;
}

void conv_forms_clear()
{
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.clear();
}

int conv_tc_autotune(const TcConvArgs &a, cudaStream_t st)
{
    if (a.mode < 0 || a.mode > 2) return fail(CNNCRF_EINVAL, "conv_tc_autotune: inference modes 0-2 only");
    // the default form first: it wins ties
    std::vector<ConvForm> cands;
    const int first_pair = g_pairs.load() != 0 ? 1 : 0;
    for (int pr : {first_pair, 1 - first_pair})
        for (int s = MAX_STAGES; s >= 2; --s) cands.push_back(ConvForm{pr, s});
    const int reps = 3;
    std::vector<cudaEvent_t> ev(cands.size() * reps * 2, nullptr);
    int rc = CNNCRF_OK;
    for (auto &e : ev)
        if (rc == CNNCRF_OK && cudaEventCreate(&e) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "conv tune: event");
    TcConvArgs b = a;
    for (int r = 0; r < reps && rc == CNNCRF_OK; ++r)
        for (size_t c = 0; c < cands.size() && rc == CNNCRF_OK; ++c) {
            b.form = cands[c];
            cudaEvent_t *e = &ev[(c * reps + r) * 2];
            if (cudaEventRecord(e[0], st) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "conv tune: record");
            if (rc == CNNCRF_OK) rc = conv_tc(b, st);
            if (rc == CNNCRF_OK && cudaEventRecord(e[1], st) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "conv tune: record");
        }
    if (rc == CNNCRF_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "conv tune: sync");
    ConvForm best = cands[0];
    float bms = 1e30f;
    for (size_t c = 0; c < cands.size() && rc == CNNCRF_OK; ++c) {
        float m = 1e30f;
        for (int r = 0; r < reps; ++r) {
            float x = 0;
            cudaEventElapsedTime(&x, ev[(c * reps + r) * 2], ev[(c * reps + r) * 2 + 1]);
            m = std::min(m, x);
        }
        if (m < bms) bms = m, best = cands[c];
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    if (rc != CNNCRF_OK) return rc;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[conv_key(a)] = ConvTuned{best, bms};
    return CNNCRF_OK;
}

int conv_tc(const TcConvArgs &a, cudaStream_t st)
{
    if (a.cp_in % 64 != 0 || a.cp_in < 64) return fail(CNNCRF_EINVAL, "conv_tc: cp_in %d not a multiple of 64", a.cp_in);
    if (a.cin < 1 || a.cin > a.cp_in) return fail(CNNCRF_EINVAL, "conv_tc: cin %d", a.cin);
    if (a.kw < 1 || a.kw > 3 || a.kh < 1) return fail(CNNCRF_EUNSUPPORTED, "conv_tc: kernel %dx%d", a.kh, a.kw);
    static_assert(AROWS - 2 * BM + 1 >= 3, "the input window covers kx shifts up to 2 for the second half");
    if (((uintptr_t)a.in & 15) || ((uintptr_t)a.wt & 15) || ((uintptr_t)a.out & 15))
        return fail(CNNCRF_EINVAL, "conv_tc: operands must be 16-byte aligned");
    TcParams p{};
    p.n_img = a.n_img, p.Hin = a.Hin, p.Win = a.Win;
    p.Ho = a.Hin - a.kh + 1, p.Wo = a.Win - a.kw + 1;
    if (p.Ho < 1 || p.Wo < 1) return fail(CNNCRF_ESHAPE, "conv_tc: empty output");
    p.kh = a.kh, p.kw = a.kw, p.cp_in = a.cp_in, p.kchunks = a.cp_in / 64;
    int rem = a.cin - 64 * (p.kchunks - 1);
    p.kk_last = rem <= 0 ? 1 : std::min(4, (rem + 15) / 16);
    p.cout = a.cout, p.cp_out = a.cp_out;
    const int rem256 = p.Wo % TILE_PX;
    if (rem256 > 0 && rem256 <= BM) { // independent halves: the last paired tile of a row would be mostly empty
        p.tiles_x = ceil_div(p.Wo, BM);
        p.halves = a.n_img * p.Ho * p.tiles_x;
        p.num_tiles = ceil_div(p.halves, 2);
        p.a_bytes = 2 * HROWS * 128;
    } else {
        p.tiles_x = ceil_div(p.Wo, TILE_PX);
        p.halves = 0;
        p.num_tiles = a.n_img * p.Ho * p.tiles_x;
        p.a_bytes = AROWS * 128;
    }
    p.mode = a.mode;
    p.bias = a.bias, p.head = a.head, p.out = a.out, p.err = a.err;
    p.aux = (const __nv_bfloat16 *)a.aux, p.out16 = a.mode >= 1 ? (__nv_bfloat16 *)a.out16 : nullptr;
    p.aux_cs = a.aux_cs, p.o16_cs = a.o16_cs, p.o16_ph = a.o16_ph, p.o16_pw = a.o16_pw;
    p.bias_part = a.mode == 4 ? a.bias_part : nullptr;
    if (a.mode != 4 && !a.out) return fail(CNNCRF_EINVAL, "conv_tc: output");
    if (a.mode < 0 || a.mode > 4) return fail(CNNCRF_EINVAL, "conv_tc: mode %d", a.mode);
    if (a.mode == 4 && (!a.aux || !a.out16 || a.aux_cs % 8 || a.aux_cs < a.np || a.o16_cs % 8 ||
                        a.o16_cs < a.np || a.o16_ph < 0 || a.o16_pw < 0 || ((uintptr_t)a.aux & 15) ||
                        ((uintptr_t)a.out16 & 15)))
        return fail(CNNCRF_EINVAL, "conv_tc: mode 4 operands");
    if ((a.mode == 1 || a.mode == 2) && a.out16 &&
        (a.o16_cs % 8 || a.o16_cs < a.np || a.o16_ph || a.o16_pw || ((uintptr_t)a.out16 & 15)))
        return fail(CNNCRF_EINVAL, "conv_tc: mode %d second output", a.mode);
    // BF16 outputs store whole 16-channel groups; FP32 input gradients float4 groups below cout
    const bool bf16_out = a.mode == 0 || a.mode == 1;
    if (bf16_out && a.cp_out % 8 != 0) return fail(CNNCRF_EINVAL, "conv_tc: cp_out %d", a.cp_out);
    if (a.mode >= 3 && (a.cp_out % 4 != 0 || a.cp_out < a.cout || a.cout > a.np))
        return fail(CNNCRF_EINVAL, "conv_tc: cp_out %d / cout %d", a.cp_out, a.cout);
    if (a.mode < 3 && !a.bias) return fail(CNNCRF_EINVAL, "conv_tc: bias");
    switch (a.np) {
    case 64:
        if (bf16_out && a.cp_out < 64) return fail(CNNCRF_EINVAL, "conv_tc: cp_out < N");
        return launch<64>(a, p, st);
    case 112:
        if (bf16_out && a.cp_out < 112) return fail(CNNCRF_EINVAL, "conv_tc: cp_out < N");
        return launch<112>(a, p, st);
    case 128:
        if (bf16_out && a.cp_out < 128) return fail(CNNCRF_EINVAL, "conv_tc: cp_out < N");
        return launch<128>(a, p, st);
    default:
        return fail(CNNCRF_EUNSUPPORTED, "conv_tc: N = %d (64, 112, 128 built)", a.np);
    }
}

} // namespace k
} // namespace cnncrf
