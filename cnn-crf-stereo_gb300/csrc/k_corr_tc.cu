// k_corr_tc.cu -- the BF16 path's correlation cost volume on the tcgen05
// tensor cores, with the unary fused into the epilogue.
//
// Replaces kCorrelation_NHWC (stereo/operators/stereocorrelation.cu:111-142,
// integer disparities, rectCorr = 0) followed by the channel softmax and the
// negation (stereo/operators/softmax.cpp:30-38, stereo/utils.cu:289-292), or
// by 1 - <fL,fR> on L2-normalised features.
//
// Banded GEMM per image row: a tile is 128 consecutive left pixels x0.. of
// row y (UMMA M = 128) against the 256 right pixels starting at x0 + omin
// (UMMA N = 256), K = the feature channels.  Left pixel m and disparity index
// k meet in band column n = m + s_k - omin (s_k = the stored, negated
// disparity), so the tile holds every product the 128 pixels need as long as
// omax - omin <= 128.  Right pixels outside [0, W) arrive as zeros through
// TMA's out-of-bounds fill: exactly the reference's 0 for w - d < 0.
//
// Wider lists (D = 192 at 1440 x 960, up to D = 516) are cut into up to four
// contiguous parts whose bands are each <= 128 wide; a tile is then (pixel
// block, part), the part's band origin moves the right-feature box, and the
// epilogue writes the part's slice of every pixel's D costs.  The parts of
// one pixel block are consecutive tiles, so the second read of its left
// features comes from L2.  The channel softmax needs all D taps of a pixel in
// one warp and so takes single-part lists only; 1 - <fL,fR> takes any.
//
// Persistent, warp-specialised CTA (576 threads, one per SM):
//   warp 0      TMA: per 64-channel block, a 4-D box (64 ch x 128 px) of the
//               left features and one (64 ch x 256 px) of the right
//               features, 128-byte swizzle; a ring of `stages` blocks
//   warp 1      TMEM allocation + single-thread tcgen05.mma (M=128, N=256,
//               K=16 steps) into one of two 256-column accumulators
//   warps 2..17 epilogue, four warps per TMEM lane quarter q = warp % 4
//               (pixels 32q..32q+31): the four read the 32 + omax - omin
//               columns those pixels touch into shared memory (one row per
//               pixel; each warp every fourth 32-column chunk), meet at a
//               named barrier, and then each warp takes every fourth pixel:
//               the whole warp gathers the pixel's D taps along the band
//               (lane j: k = j + 32 r), applies the unary and stores its D
//               costs with coalesced writes.  Sixteen warps instead of four
//               hide the gather's latency; the four agree on every exit so
//               none waits at the barrier for a partner that left.
// Every mbarrier wait is bounded; on timeout the role raises the CTA abort
// flag and the global error flag, drains what it issued and TMEM is freed.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include <cuda.h>
#include <cuda_bf16.h>

#include "../../include/cnncrf_fmath.h"
#include "common.h"
#include "kernels.h"
#include "tc_util.cuh"

namespace cnncrf {
namespace k {

namespace {

constexpr int BM = 128;                    // left pixels per tile (UMMA M)
constexpr int BN = 256;                    // band columns per tile (UMMA N)
constexpr int A_BYTES = BM * 128;          // 128 px x 64 bf16
constexpr int B_BYTES = BN * 128;          // 256 px x 64 bf16
constexpr int STAGE = A_BYTES + B_BYTES;   // one 64-channel block of a tile
// epilogue warps per TMEM lane quarter.  Per KITTI step of 8 pairs the kernel
// took 1.13 ms with 1, 0.80 with 2, 0.73 with 3 and 0.70 with 4 (GB300)
constexpr int EPI_WARPS = 4;
constexpr uint32_t TMEM_COLS = 2 * BN;     // two accumulators
constexpr int SROW = 161;                  // staged row stride in floats (odd: no bank conflicts)
constexpr int SCOLS = 160;                 // columns staged per warp: 32 + max band spread
constexpr int MAXP = 8;                    // taps per lane: <= 256 disparities per part
constexpr int MAXPARTS = 4;                // disparity parts of a wide list
constexpr int STG_BYTES = 4 * 32 * SROW * 4;
constexpr uint32_t IDESC = tc::idesc_bf16(BM, BN);

struct CorrTcParams {
    int H, W, npairs, D, nkb, kk_last, tiles_x, num_tiles, unary, stages, nparts;
    int pk0[MAXPARTS], pD[MAXPARTS], pomin[MAXPARTS], pnch[MAXPARTS]; // per part: first k, count, band origin, chunks
    const float *list;
    float *out;        // the FP32 volume (null: not written)
    uint16_t *outq;    // optional 16-bit fixed-point copy (the BF16 path's CRF unary), same layout
    float qinv, qbias; // q = x / scale - offset / scale rounded to the nearest integer, saturated to 0..65535
    int *err;
};

// x * qinv is exact (qinv a power of two), so the FMA rounds once, like the
// product plus qbias in FP32; the conversion rounds to nearest-even and saturates
__device__ __forceinline__ uint16_t quantize_u16(float x, float qinv, float qbias)
{
    unsigned short q;
    asm("cvt.rni.sat.u16.f32 %0, %1;" : "=h"(q) : "f"(__fmaf_rn(x, qinv, qbias)));
    return q;
}

// The epilogue's per-pixel part for PP taps per lane (a part of Dp <= 32 PP
// disparities): each pixel's band diagonal from the warp's staged rows, the
// unary, and the stores: the FP32 volume (WF) and / or its 16-bit copy (WQ),
// chosen at compile time so the per-element stores carry no branches.
template <int EPW, int PP, bool WF, bool WQ>
__device__ __forceinline__ void store_pixels(const CorrTcParams &p, const float *sw, int lane, int i0, int npx,
                                             int Dp, const int *off, float *obase, uint16_t *obaseq)
{
#pragma unroll 1
    for (int i = i0; i < npx; i += EPW) {
        const float *row = sw + i * SROW + i;
        float cv[PP];
#pragma unroll
        for (int rr = 0; rr < PP; ++rr) cv[rr] = (lane + 32 * rr < Dp) ? row[off[rr]] : 0.0f;
        float *o = WF ? obase + (size_t)i * p.D : nullptr;
        uint16_t *oq = WQ ? obaseq + (size_t)i * p.D : nullptr;
        if (p.unary == 0) {
            float m = -FLT_MAX;
#pragma unroll
            for (int rr = 0; rr < PP; ++rr)
                if (lane + 32 * rr < Dp) m = fmaxf(m, cv[rr]);
#pragma unroll
            for (int s = 16; s >= 1; s >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, s));
            float sum = 0.0f;
#pragma unroll
            for (int rr = 0; rr < PP; ++rr) {
                const float e = lane + 32 * rr < Dp ? cnncrf_expf(cv[rr] - m) : 0.0f;
                cv[rr] = e;
                sum = (rr == 0) ? e : sum + e;
            }
#pragma unroll
            for (int s = 16; s >= 1; s >>= 1) sum = sum + __shfl_xor_sync(0xffffffffu, sum, s);
#pragma unroll
            for (int rr = 0; rr < PP; ++rr) {
                const int kk = lane + 32 * rr;
                if (kk < Dp) {
                    const float u = -(cv[rr] / sum);
                    if constexpr (WF) o[kk] = u;
                    if constexpr (WQ) oq[kk] = quantize_u16(u, p.qinv, p.qbias);
                }
            }
        } else {
#pragma unroll
            for (int rr = 0; rr < PP; ++rr) {
                const int kk = lane + 32 * rr;
                if (kk < Dp) {
                    const float u = p.unary == 1 ? 1.0f - cv[rr] : cv[rr];
                    if constexpr (WF) o[kk] = u;
                    if constexpr (WQ) oq[kk] = quantize_u16(u, p.qinv, p.qbias);
                }
            }
        }
    }
}

// pixels i0, i0 + EPW, ... of the warp's 32 (the EPW warps of a lane quarter split them)
template <int EPW, bool WF, bool WQ>
__device__ __forceinline__ void store_part(const CorrTcParams &p, int P, const float *sw, int lane, int i0, int npx,
                                           int Dp, const int *off, float *obase, uint16_t *obaseq)
{
    switch (P) {
    case 1: store_pixels<EPW, 1, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    case 2: store_pixels<EPW, 2, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    case 3: store_pixels<EPW, 3, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    case 4: store_pixels<EPW, 4, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    case 5: store_pixels<EPW, 5, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    case 6: store_pixels<EPW, 6, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    case 7: store_pixels<EPW, 7, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    default: store_pixels<EPW, 8, WF, WQ>(p, sw, lane, i0, npx, Dp, off, obase, obaseq); break;
    }
}

template <int EPW>
__global__ void __launch_bounds__(64 + 128 * EPW, 1)
    k_corr_tc(const __grid_constant__ CUtensorMap tmL, const __grid_constant__ CUtensorMap tmR, const CorrTcParams p)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = p.stages;
    float *stg = (float *)(smem + S * STAGE);
    uint64_t *full = (uint64_t *)((uint8_t *)stg + STG_BYTES);
    uint64_t *empty = full + S;
    uint64_t *tfull = empty + S;
    uint64_t *tempty = tfull + 2;
    uint64_t *drain = tempty + 2;
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    volatile int *zero_flag = abort_flag + 1;
    int *coff = (int *)(tmem_slot + 4); // [D] band column offset of disparity k
    volatile int *okq = (volatile int *)(coff + p.D); // [4][EPW] each epilogue warp's tfull wait result
    constexpr int NUM_THREADS = 64 + 128 * EPW;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], 128 * EPW);
        }
        tc::mbar_init(drain, 1);
        *abort_flag = 0;
        *zero_flag = 0;
        tc::mbar_fence_init();
        tc::prefetch_tmap(&tmL);
        tc::prefetch_tmap(&tmR);
    }
    for (int pp = 0; pp < p.nparts; ++pp) // band column of disparity k within its part's tile
        for (int i = threadIdx.x; i < p.pD[pp]; i += NUM_THREADS)
            coff[p.pk0[pp] + i] = (int)p.list[p.pk0[pp] + i] - p.pomin[pp];
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const int tiles_per_pair = p.H * p.tiles_x;

    if (warp == 0) {
        if (lane == 0) {
            int stage = 0, issued = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < p.num_tiles && ok; t += gridDim.x) {
                const int part = t % p.nparts, tt = t / p.nparts;
                const int pair = tt / tiles_per_pair, r = tt - pair * tiles_per_pair;
                const int y = r / p.tiles_x, x0 = (r - y * p.tiles_x) * BM;
                for (int kb = 0; kb < p.nkb; ++kb) {
                    if (!tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    uint8_t *sa = smem + stage * STAGE;
                    tc::mbar_expect_tx(&full[stage], STAGE);
                    tc::tma_load_4d(sa, &tmL, &full[stage], kb * 64, x0, y, pair);
                    tc::tma_load_4d(sa + A_BYTES, &tmR, &full[stage], kb * 64, x0 + p.pomin[part], y,
                                    p.npairs + pair);
                    ++issued;
                    if (++stage == S) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
            }
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
                // let the copies already issued land before shared memory is released
                int st = stage;
                uint32_t ph = phase;
                for (int i = 0; i < S && i < issued; ++i) {
                    if (--st < 0) {
                        st = S - 1;
                        ph ^= 1;
                    }
                    tc::mbar_wait(&full[st], ph, zero_flag, 1u << 20);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            int stage = 0, lt = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < p.num_tiles && ok; t += gridDim.x, ++lt) {
                const int buf = lt & 1;
                const uint32_t use = (uint32_t)lt >> 1;
                if (!tc::mbar_wait(&tempty[buf], (use & 1) ^ 1, abort_flag)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t d = tmem + buf * BN;
                for (int kb = 0; kb < p.nkb; ++kb) {
                    if (!tc::mbar_wait(&full[stage], phase, abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const int nk = (kb == p.nkb - 1) ? p.kk_last : 4;
                    const uint32_t sa = tc::smem_u32(smem + stage * STAGE);
                    const uint64_t da = tc::sdesc_sw128(sa), db = tc::sdesc_sw128(sa + A_BYTES);
                    for (int kk = 0; kk < nk; ++kk)
                        tc::umma_bf16(d, da + 2 * kk, db + 2 * kk, IDESC, (kb | kk) != 0 ? 1u : 0u);
                    tc::umma_commit(&empty[stage]);
                    if (++stage == S) {
                        stage = 0;
                        phase ^= 1;
                    }
                }
                if (ok) tc::umma_commit(&tfull[buf]);
            }
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
            }
            // every MMA of this thread completes before TMEM is released
            tc::umma_commit(drain);
            tc::mbar_wait(drain, 0, zero_flag, 1u << 22);
        }
    } else {
        const int q = warp & 3;         // the TMEM lane quarter this warp may read
        const int h = (warp - 2) >> 2;  // which of the quarter's EPW warps
        float *sw = stg + q * 32 * SROW;
        int lt = 0;
        for (int t = blockIdx.x; t < p.num_tiles; t += gridDim.x, ++lt) {
            const int part = t % p.nparts, tt = t / p.nparts;
            const int Dp = p.pD[part], k0 = p.pk0[part];
            const int P = (Dp + 31) >> 5;
            int off[MAXP];
#pragma unroll
            for (int r = 0; r < MAXP; ++r) {
                const int kk = lane + 32 * r;
                off[r] = (r < P && kk < Dp) ? coff[k0 + kk] : 0;
            }
            const int buf = lt & 1;
            const uint32_t use = (uint32_t)lt >> 1;
            // both warps wait (bounded) and publish the result; both then act on
            // the pair's combined result, so they leave the loop together
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&tfull[buf], use & 1, abort_flag) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (lane == 0) okq[EPW * q + h] = ok;
            // the pair's barrier: both results published, and the partner is done
            // gathering from the staged rows of the previous tile
            asm volatile("bar.sync %0, %1;" ::"r"(1 + q), "n"(32 * EPW) : "memory");
#pragma unroll
            for (int e = 0; e < EPW; ++e) ok &= okq[EPW * q + e];
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
                break;
            }
            tc::fence_after_sync();
            // rows 32q.. of the accumulator, columns 32q .. 32q + 32*nchunks; this warp's chunks h, h + 2, ..
            const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + buf * BN + q * 32;
            float v[32];
#pragma unroll 1
            for (int c = h; c < p.pnch[part]; c += EPW) {
                tc::tmem_ld32(ta + c * 32, v); // warp-collective: every lane runs it
#pragma unroll
                for (int j = 0; j < 32; ++j) sw[lane * SROW + c * 32 + j] = v[j];
            }
            tc::fence_before_sync();
            tc::mbar_arrive(&tempty[buf]);
            asm volatile("bar.sync %0, %1;" ::"r"(1 + q), "n"(32 * EPW) : "memory"); // all chunks staged

            const int pair = tt / tiles_per_pair, r = tt - pair * tiles_per_pair;
            const int y = r / p.tiles_x, xq = (r - y * p.tiles_x) * BM + q * 32;
            const int npx = min(32, p.W - xq);
            const size_t obase_i = (((size_t)pair * p.H + y) * p.W + xq) * p.D + k0;
            float *obase = p.out ? p.out + obase_i : nullptr;
            uint16_t *obaseq = p.outq ? p.outq + obase_i : nullptr;
            if (obaseq && obase) store_part<EPW, true, true>(p, P, sw, lane, h, npx, Dp, off, obase, obaseq);
            else if (obaseq) store_part<EPW, false, true>(p, P, sw, lane, h, npx, Dp, off, obase, obaseq);
            else store_part<EPW, true, false>(p, P, sw, lane, h, npx, Dp, off, obase, obaseq);
            // the next tile's first barrier keeps its staging behind the partner's gather
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

size_t smem_bytes(int stages, int D)
{
    return 1024 + (size_t)stages * STAGE + STG_BYTES + (2 * (size_t)stages + 5) * 8 + 16 + (size_t)D * 4 + 64;
}

struct CorrTcPlan {
    int nparts = 0;
    int k0[MAXPARTS], D[MAXPARTS], omin[MAXPARTS], omax[MAXPARTS];
};

// The fewest near-equal contiguous parts of the stored list whose bands each
// fit a tile (band spread <= BN - BM); false if the list has a fractional
// entry, needs more than MAXPARTS parts, or needs several under the softmax.
bool corr_tc_plan(const float *h_list, int D, int unary, CorrTcPlan &pl)
{
    if (!h_list || D < 1 || D > MAXPARTS * (BN - BM + 1)) return false;
    for (int i = 0; i < D; ++i)
        if (h_list[i] != std::floor(h_list[i]) || std::fabs(h_list[i]) > (float)(1 << 20)) return false;
    for (int np = 1; np <= MAXPARTS && (np == 1 || unary != 0); ++np) {
        if (np > D) break;
        bool ok = D / np + 1 <= 32 * MAXP; // a part's taps fit the epilogue's registers
        int k0 = 0;
        for (int pp = 0; pp < np && ok; ++pp) {
            const int n = D / np + (pp < D % np ? 1 : 0);
            int lo = 1 << 30, hi = -(1 << 30);
            for (int i = k0; i < k0 + n; ++i) {
                lo = std::min(lo, (int)h_list[i]);
                hi = std::max(hi, (int)h_list[i]);
            }
            ok = hi - lo <= BN - BM && 32 + (hi - lo) <= SCOLS;
            pl.k0[pp] = k0, pl.D[pp] = n, pl.omin[pp] = lo, pl.omax[pp] = hi;
            k0 += n;
        }
        if (ok) {
            pl.nparts = np;
            return true;
        }
    }
    return false;
}

} // namespace

bool unary_q16(int unary, UnaryQ16 *q)
{
    if (unary == 1) { // 1 - cosine in [0, 2] (a little outside where BF16 rounding lifts |cos| past 1)
        q->scale = 1.0f / 32768.0f, q->offset = -1.0f / 256.0f;
    } else if (unary == 0) { // -softmax in [-1, 0]
        q->scale = 1.0f / 65536.0f, q->offset = -1.0f;
    } else {
        return false;
    }
    // the CRF's dequantisation computes (2^23 + q) scale + (offset - 2^23 scale):
    // that offset must be exact in FP32 (it is for both codes above)
    return (double)(q->offset - 8388608.0f * q->scale) == (double)q->offset - 8388608.0 * (double)q->scale;
}

bool corr_tc_supported(int C, int cp, const float *h_list, int D, int unary)
{
    CorrTcPlan pl;
    return cp % 64 == 0 && C >= 1 && C <= cp && corr_tc_plan(h_list, D, unary, pl);
}

int correlation_tc(const void *feat, int npairs, int H, int W, int C, int cp, const float *d_list,
                   const float *h_list, int D, int unary, float *out, int *err, cudaStream_t st, void *outq)
{
    CorrTcPlan pl;
    if (!(cp % 64 == 0 && C >= 1 && C <= cp) || !corr_tc_plan(h_list, D, unary, pl))
        return fail(CNNCRF_EUNSUPPORTED, "correlation_tc: C=%d cp=%d D=%d unary %d", C, cp, D, unary);
    if (npairs < 1 || H < 1 || W < 1) return fail(CNNCRF_EINVAL, "correlation_tc: bad size");
    if (((uintptr_t)feat & 15) || (!out && !outq) || !err || !d_list)
        return fail(CNNCRF_EINVAL, "correlation_tc: bad pointer");
    UnaryQ16 uq{1.0f, 0.0f};
    if (outq && !unary_q16(unary, &uq))
        return fail(CNNCRF_EUNSUPPORTED, "correlation_tc: no 16-bit copy of unary %d", unary);
    auto enc = tc::tensor_map_encoder();
    if (!enc) return fail(CNNCRF_ECUDA, "correlation_tc: cuTensorMapEncodeTiled unavailable");
    // features [2 * npairs][H][W][cp] BF16: left images first, then right images
    cuuint64_t g[4] = {(cuuint64_t)cp, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)(2 * npairs)};
    cuuint64_t s[3] = {(cuuint64_t)cp * 2, (cuuint64_t)W * cp * 2, (cuuint64_t)H * W * cp * 2};
    cuuint32_t e[4] = {1, 1, 1, 1};
    cuuint32_t bl[4] = {64, BM, 1, 1};
    cuuint32_t br[4] = {64, BN, 1, 1};
    CUtensorMap ml, mr;
    CUresult r = enc(&ml, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)feat, g, s, bl, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "correlation_tc: left tensor map (%d)", (int)r);
    r = enc(&mr, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)feat, g, s, br, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "correlation_tc: right tensor map (%d)", (int)r);

    CorrTcParams p{};
    p.H = H, p.W = W, p.npairs = npairs, p.D = D;
    p.nkb = ceil_div(C, 64);
    p.kk_last = ceil_div(C - 64 * (p.nkb - 1), 16);
    p.nparts = pl.nparts;
    for (int pp = 0; pp < pl.nparts; ++pp) {
        p.pk0[pp] = pl.k0[pp], p.pD[pp] = pl.D[pp], p.pomin[pp] = pl.omin[pp];
        p.pnch[pp] = ceil_div(32 + (pl.omax[pp] - pl.omin[pp]), 32);
    }
    p.tiles_x = ceil_div(W, BM);
    p.num_tiles = npairs * H * p.tiles_x * pl.nparts;
    p.unary = unary;
    p.list = d_list, p.out = out, p.outq = (uint16_t *)outq, p.err = err;
    p.qinv = 1.0f / uq.scale, p.qbias = -uq.offset / uq.scale;

    int dev = 0, sms = 0, maxsm = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    p.stages = smem_bytes(3, D) <= (size_t)maxsm ? 3 : 2;
    const size_t smem = smem_bytes(p.stages, D);
    if (smem > (size_t)maxsm) return fail(CNNCRF_EUNSUPPORTED, "correlation_tc: %zu bytes of shared memory", smem);
    auto kern = k_corr_tc<EPI_WARPS>;
    CNNCRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = std::min(p.num_tiles, sms);
    {
        CNNCRF_PROF("corr_tc", st);
        kern<<<grid, 64 + 128 * EPI_WARPS, smem, st>>>(ml, mr, p);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
