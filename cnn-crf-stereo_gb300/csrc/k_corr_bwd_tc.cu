// k_corr_bwd_tc.cu -- the adjoint of the one-minus-dot correlation
// (vol[u][k] = 1 - <fl[u], fr[u + s_k]>, s_k the stored list) on the tcgen05
// tensor cores, for the BF16 training step:
//
//   dF[u][c] = -sum_v A[u][v] P[v][c],   A[u][v] = a(u, k) where v = u + o_k
//
//   left  (dF = dfl): P = fr, o_k =  s_k, a(u, k) = gvol[u][k]
//   right (dF = dfr): P = fl, o_k = -s_k, a(u, k) = gvol[u - s_k][k] = gvol[v][k]
//
// A tile is 128 output pixels u of one row; v runs over the window
// x0 + omn .. x0 + omn + 127 + span - 1 (omn = min o_k, span = max o_k -
// omn + 1) in K-blocks of 64 pixels.  The builder warps first copy the
// tile's volume-gradient rows to shared memory as BF16 with coalesced loads
// (left: the 128 rows u; right: the window rows v), then write, per K-block,
// one shared-memory stage of
//   A [128 u][64 v] BF16, K-major 128-byte swizzle: row u holds a(u, k) at
//     v - u = o_k and zeros elsewhere
// while TMA brings
//   P [64 v][C] BF16 from NHWC: MN-major, a box per 64 channels.
// Warps: 0 TMA; 1 TMEM allocation + single-thread tcgen05.mma (M = 128,
// N = NP, K = 16 x 4 per block; A K-major, B MN-major); 2..9 builders (two
// threads per A row, four 16-byte chunks each); 10..13 epilogue (TMEM ->
// -sum -> FP32 NHWC).  Two TMEM
// accumulators: the epilogue of tile i overlaps tile i + 1.  Every mbarrier
// wait is bounded; on timeout the roles raise the abort and error flags,
// drain and free TMEM.  The offsets of the list must be distinct.
#include <algorithm>

#include <cuda.h>
#include <cuda_bf16.h>

#include "common.h"
#include "kernels.h"
#include "tc_util.cuh"

namespace cnncrf {
namespace k {

namespace {

constexpr int BM = 128;                // output pixels per tile (UMMA M)
constexpr int KB = 64;                 // window pixels per K-block
constexpr int A_BYTES = BM * 128;      // 16 KB
constexpr int P_BOX = 64 * KB * 2;     // one 64-channel x 64-pixel box: 8 KB
constexpr int STAGE_BYTES = A_BYTES + 2 * P_BOX;
constexpr int NB = 8;                             // builder warps
constexpr int NUM_THREADS = 32 * (2 + NB + 4);
constexpr uint32_t TMEM_COLS = 256;    // two accumulators of 128 columns
constexpr int MAX_STAGES = 6;
constexpr int MAX_SPAN = 1024;

struct CbParams {
    const float *g;    // [npairs][H][W][D]: the volume gradient
    const float *list; // the stored list s_k
    float *out;        // [npairs][H][W][C]
    int H, W, C, D, np, p_boxes, right, omn, span, nkb, tiles_x, num_tiles, stages, grows, gstride;
    int *err;
};

__device__ __forceinline__ void st_shared_v4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d)
{
    asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *(uint32_t *)&h;
}

__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_corr_bwd_tc(const __grid_constant__ CUtensorMap tmP, const CbParams p)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = p.stages;
    uint64_t *full = (uint64_t *)(smem + S * STAGE_BYTES);
    uint64_t *empty = full + S;
    uint64_t *tfull = empty + S;
    uint64_t *tempty = tfull + 2;
    uint64_t *drain = tempty + 2;
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    volatile int *zero_flag = abort_flag + 1;
    short *inv = (short *)(tmem_slot + 4); // [span]: k with o_k = omn + i, or -1
    // the tile's volume-gradient rows, BF16 [grows][gstride] (16-byte aligned rows)
    __nv_bfloat16 *gs = (__nv_bfloat16 *)(((uintptr_t)(inv + p.span) + 15) & ~(uintptr_t)15);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            tc::mbar_init(&full[s], 1 + NB); // the TMA producer's expect_tx + one arrival per builder warp
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], 128);
        }
        tc::mbar_init(drain, 1);
        *abort_flag = 0;
        *zero_flag = 0;
        tc::mbar_fence_init();
        tc::prefetch_tmap(&tmP);
    }
    for (int i = threadIdx.x; i < p.span; i += NUM_THREADS) inv[i] = -1;
    __syncthreads();
    for (int k = threadIdx.x; k < p.D; k += NUM_THREADS)
        inv[(p.right ? -(int)p.list[k] : (int)p.list[k]) - p.omn] = (short)k;
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const int per_img = p.H * p.tiles_x;

    if (warp == 0) {
        if (lane == 0) {
            int stage = 0, issued = 0;
            uint32_t phase = 0;
            bool ok = true;
            const uint32_t tx = (uint32_t)p.p_boxes * P_BOX;
            for (int t = blockIdx.x; t < p.num_tiles && ok; t += gridDim.x) {
                const int pair = t / per_img, r = t - pair * per_img;
                const int y = r / p.tiles_x, x0 = (r - y * p.tiles_x) * BM;
                for (int kb = 0; kb < p.nkb; ++kb) {
                    if (!tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
                        ok = false;
                        break;
                    }
                    uint8_t *sp = smem + stage * STAGE_BYTES + A_BYTES;
                    tc::mbar_expect_tx(&full[stage], tx);
                    for (int b = 0; b < p.p_boxes; ++b)
                        tc::tma_load_4d(sp + b * P_BOX, &tmP, &full[stage], b * 64, x0 + p.omn + kb * KB, y, pair);
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
                int st = stage;
                uint32_t ph = phase;
                for (int i = 0; i < S && i < issued; ++i) {
                    if (--st < 0) {
                        st = S - 1;
                        ph ^= 1;
                    }
                    // the builders' arrivals may never come: wait for the copies alone (bounded)
                    tc::mbar_wait(&full[st], ph, zero_flag, 1u << 20);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // B (P) MN-major: the transpose-B bit; A K-major
            const uint32_t idesc = tc::idesc_bf16(BM, p.np) | (1u << 16);
            int stage = 0, lt = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < p.num_tiles && ok; t += gridDim.x, ++lt) {
                const int buf = lt & 1;
                if (!tc::mbar_wait(&tempty[buf], (((uint32_t)lt >> 1) & 1u) ^ 1u, abort_flag)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t d = tmem + buf * 128;
                for (int kb = 0; kb < p.nkb; ++kb) {
                    if (!tc::mbar_wait(&full[stage], phase, abort_flag)) {
                        ok = false;
                        break;
                    }
                    tc::fence_after_sync();
                    const uint32_t sa = tc::smem_u32(smem + stage * STAGE_BYTES);
                    const uint64_t da = tc::sdesc_sw128(sa);
#pragma unroll
                    for (int kk = 0; kk < KB / 16; ++kk) {
                        const uint64_t db = tc::sdesc_sw128_mn(sa + A_BYTES + kk * 2048, P_BOX);
                        tc::umma_bf16(d, da + 2 * kk, db, idesc, (kb | kk) ? 1u : 0u);
                    }
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
            tc::umma_commit(drain);
            tc::mbar_wait(drain, 0, zero_flag, 1u << 22);
        }
    } else if (warp < 2 + NB) {
        // builders: threads r and r + 128 write row r (output pixel x0 + r) of every K-block's A,
        // chunks 0..3 and 4..7
        const int bw = warp - 2, bt = bw * 32 + lane, r = bt & (BM - 1), jh = (bt >> 7) * 4;
        // A warp whose wait gave up keeps looping without work: the four builder
        // warps pass the named barrier below the same number of times.
        int stage = 0;
        uint32_t phase = 0;
        bool ok = true;
        const bool vec = (p.D & 3) == 0; // 16-byte aligned gradient rows
        for (int t = blockIdx.x; t < p.num_tiles; t += gridDim.x) {
            const int pair = t / per_img, rr = t - pair * per_img;
            const int y = rr / p.tiles_x, x0 = (rr - y * p.tiles_x) * BM;
            const bool rowvalid = x0 + r < p.W;
            // 1. the gradient rows: left pixels x0 + i, right pixels x0 + omn + i; zero outside the row
            const long rowbase = ((long)pair * p.H + y) * p.W;
            const int g0 = p.right ? x0 + p.omn : x0;
            asm volatile("bar.sync 1, %0;" ::"n"(32 * NB) : "memory"); // the previous tile's reads are done
            // 16 rows in flight per warp: lane l holds channels 4l .. 4l + 3 of a 128-wide column chunk
            for (int kc = 0; kc < p.D && ok; kc += 128) {
                const int k = kc + 4 * lane;
                for (int i0 = bw; i0 < p.grows; i0 += 16 * NB) {
                    float4 v[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int i = i0 + NB * q, x = g0 + i;
                        v[q] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        if (i < p.grows && x >= 0 && x < p.W && k < p.D) {
                            const float *src = p.g + (rowbase + x) * p.D + k;
                            if (vec) {
                                v[q] = __ldg((const float4 *)src);
                            } else {
                                v[q].x = __ldg(src);
                                v[q].y = k + 1 < p.D ? __ldg(src + 1) : 0.0f;
                                v[q].z = k + 2 < p.D ? __ldg(src + 2) : 0.0f;
                                v[q].w = k + 3 < p.D ? __ldg(src + 3) : 0.0f;
                            }
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const int i = i0 + NB * q;
                        if (i < p.grows && k < p.D)
                            *(uint2 *)(gs + (long)i * p.gstride + k) =
                                make_uint2(pack_bf16(v[q].x, v[q].y), pack_bf16(v[q].z, v[q].w));
                    }
                }
            }
            asm volatile("bar.sync 1, %0;" ::"n"(32 * NB) : "memory");
            for (int kb = 0; kb < p.nkb && ok; ++kb) {
                int got = 1;
                if (lane == 0) got = tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag) ? 1 : 0;
                got = __shfl_sync(0xffffffffu, got, 0);
                if (!got) {
                    ok = false;
                    break;
                }
                const uint32_t row = tc::smem_u32(smem + stage * STAGE_BYTES) + r * 128;
#pragma unroll 1
                for (int j = jh; j < jh + 4; ++j) {
                    const int i0 = kb * KB + 8 * j - r; // band index of the chunk's first pixel
                    uint32_t w[4] = {0u, 0u, 0u, 0u};
                    if (rowvalid && i0 + 7 >= 0 && i0 < p.span) {
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            float f[2];
#pragma unroll
                            for (int h = 0; h < 2; ++h) {
                                const int i = i0 + 2 * e + h;
                                const int k = (i >= 0 && i < p.span) ? inv[i] : -1;
                                // left: row r of the copy; right: row v - (x0 + omn) = the chunk's pixel
                                const int gr = p.right ? i + r : r;
                                f[h] = k >= 0 ? __bfloat162float(gs[(long)gr * p.gstride + k]) : 0.0f;
                            }
                            w[e] = pack_bf16(f[0], f[1]);
                        }
                    }
                    st_shared_v4(row + ((j ^ (r & 7)) << 4), w[0], w[1], w[2], w[3]);
                }
                // the tensor core reads A through the async proxy
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) tc::mbar_arrive(&full[stage]);
                if (++stage == S) {
                    stage = 0;
                    phase ^= 1;
                }
            }
        }
        if (!ok) {
            *abort_flag = 1;
            atomicExch(p.err, 1);
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31
        const int q = warp & 3, row = q * 32 + lane;
        int lt = 0;
        for (int t = blockIdx.x; t < p.num_tiles; t += gridDim.x, ++lt) {
            const int buf = lt & 1;
            int ok = 1;
            if (lane == 0) ok = tc::mbar_wait(&tfull[buf], ((uint32_t)lt >> 1) & 1u, abort_flag) ? 1 : 0;
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                *abort_flag = 1;
                atomicExch(p.err, 1);
                break;
            }
            tc::fence_after_sync();
            const int pair = t / per_img, rr = t - pair * per_img;
            const int y = rr / p.tiles_x, u = (rr - y * p.tiles_x) * BM + row;
            const bool valid = u < p.W;
            float *o = p.out + (((long)pair * p.H + y) * p.W + (valid ? u : 0)) * p.C;
            const bool vec4 = (p.C & 3) == 0; // 16-byte aligned output rows
            for (int c = 0; c < p.np / 16; ++c) {
                float v[16];
                tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + buf * 128 + c * 16, v); // warp-collective
                if (valid) {
#pragma unroll
                    for (int g4 = 0; g4 < 4; ++g4) {
                        const int c0 = c * 16 + 4 * g4;
                        if (vec4 && c0 + 3 < p.C)
                            *(float4 *)(o + c0) = make_float4(-v[4 * g4], -v[4 * g4 + 1], -v[4 * g4 + 2],
                                                              -v[4 * g4 + 3]);
                        else
#pragma unroll
                            for (int j = 0; j < 4; ++j)
                                if (c0 + j < p.C) o[c0 + j] = -v[4 * g4 + j];
                    }
                }
            }
            tc::fence_before_sync();
            tc::mbar_arrive(&tempty[buf]);
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

size_t smem_bytes(int stages, int span, int grows, int gstride)
{
    return 1024 + (size_t)stages * STAGE_BYTES + (2 * stages + 5) * 8 + 16 + 2 * (size_t)span + 16 +
           2 * (size_t)grows * gstride;
}

int launch_side(const void *P, int fs, const float *g, const float *d_list, int npairs, int H, int W, int C, int D,
                int right, int omn, int span, float *out, int *err, cudaStream_t st)
{
    auto enc = tc::tensor_map_encoder();
    if (!enc) return fail(CNNCRF_ECUDA, "corr_bwd_tc: cuTensorMapEncodeTiled unavailable");
    CUtensorMap mp;
    cuuint64_t gd[4] = {(cuuint64_t)fs, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)npairs};
    cuuint64_t sd[3] = {(cuuint64_t)fs * 2, (cuuint64_t)W * fs * 2, (cuuint64_t)H * W * fs * 2};
    cuuint32_t box[4] = {64, KB, 1, 1}, e[4] = {1, 1, 1, 1};
    CUresult r = enc(&mp, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)P, gd, sd, box, e,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "corr_bwd_tc: feature tensor map (%d)", (int)r);
    CbParams p{};
    p.g = g, p.list = d_list, p.out = out, p.err = err;
    p.H = H, p.W = W, p.C = C, p.D = D, p.np = (C + 15) & ~15, p.right = right, p.omn = omn, p.span = span;
    p.grows = right ? BM - 1 + span : BM;
    p.gstride = (D + 7) & ~7; // BF16 rows of whole 16-byte units
    p.p_boxes = p.np > 64 ? 2 : 1;
    p.nkb = ceil_div(BM - 1 + span, KB);
    p.tiles_x = ceil_div(W, BM);
    p.num_tiles = npairs * H * p.tiles_x;
    int dev = 0, sms = 0, maxsm = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    p.stages = 0;
    for (int s = 2; s <= MAX_STAGES; ++s)
        if (smem_bytes(s, span, p.grows, p.gstride) <= (size_t)maxsm) p.stages = s;
    if (!p.stages) return fail(CNNCRF_EUNSUPPORTED, "corr_bwd_tc: shared memory");
    const size_t smem = smem_bytes(p.stages, span, p.grows, p.gstride);
    CNNCRF_CUDA(cudaFuncSetAttribute(k_corr_bwd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_corr_bwd_tc<<<std::min(p.num_tiles, sms), NUM_THREADS, smem, st>>>(mp, p);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace

bool corr_bwd_tc_supported(int C, int fs, int D, int omin, int omax)
{
    const int span = omax - omin + 1, gstride = (D + 7) & ~7;
    // two stages beside the right side's gradient window
    return C >= 1 && C <= 128 && fs % 64 == 0 && fs >= ((C + 15) & ~15) && D >= 1 && D <= 32767 &&
           span <= MAX_SPAN && smem_bytes(2, span, BM - 1 + span, gstride) <= 227 * 1024;
}

int corr_bwd_tc(const void *fl, const void *fr, int fs, const float *gvol, const float *d_list, int npairs, int H,
                int W, int C, int D, int omin, int omax, float *dfl, float *dfr, int *err, cudaStream_t st)
{
    if (!corr_bwd_tc_supported(C, fs, D, omin, omax)) return fail(CNNCRF_EUNSUPPORTED, "corr_bwd_tc: shape");
    if (((uintptr_t)fl & 15) || ((uintptr_t)fr & 15)) return fail(CNNCRF_EINVAL, "corr_bwd_tc: feature alignment");
    const int span = omax - omin + 1;
    CNNCRF_PROF("corr_bwd", st);
    CNNCRF_TRY(launch_side(fr, fs, gvol, d_list, npairs, H, W, C, D, 0, omin, span, dfl, err, st));
    return launch_side(fl, fs, gvol, d_list, npairs, H, W, C, D, 1, -omax, span, dfr, err, st);
}

} // namespace k
} // namespace cnncrf
