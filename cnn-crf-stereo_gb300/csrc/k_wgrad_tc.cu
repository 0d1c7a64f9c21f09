// k_wgrad_tc.cu -- the weight gradient of a kh x kw convolution layer on the
// tcgen05 tensor cores (training step, BF16 mode): BF16 operands, FP32
// accumulation in TMEM.
//
//   dW'[co][ky][kx][ci] = sum over pixels p = (img, oy, ox) of
//                         dz[p][co] * x[img][oy + ky][ox + kx][ci]
//
// is a GEMM per tap with M = output channels, N = input channels and K = the
// pixels.  Both operands are read as they lie in memory, channels innermost
// (NHWC), which makes them MN-major: a TMA box of 64 channels x 64 pixels
// lands as 64 rows (one per pixel, K) of 128 bytes (64 channels, MN) in the
// 128-byte swizzle, and a second box holds channels 64..127.
//   A: the output gradient dz in its BF16 copy with a zero border of kh - 1
//      rows and kw - 1 columns ([img][Ho + 2(kh-1)][Wo + 2(kw-1)][cpa]), read
//      at (oy + kh - 1, ox + kw - 1): pixels past the row end read the border
//      or the box's zero fill, so they add nothing;
//   B: the layer input of row oy + ky, pixels x0 .. x0 + 71 (64 + a halo of
//      8) in one box per 64 channels; tap kx reads it through a descriptor
//      that starts kx 128-byte rows (pixels) in, so the input is loaded once
//      per kernel row, not once per tap.
// Channels past Cout / Cin give rows / columns of dW' that are not stored.
//
// One CTA per (ky, pixel split), 192 threads:
//   warp 0      TMA: per K step (64 pixels of one output row) the dz boxes
//               and the input boxes into a ring of stages
//   warp 1      TMEM allocation + single-thread tcgen05.mma, M = 128, N = NP,
//               K = 16 x 4 per step, into kw accumulators of 128 columns
//   warps 2..5  epilogue: warp q reads TMEM lanes (output channels) 32q..32q+31
//               of every accumulator and writes the split's FP32 partials
// A reduction kernel adds the splits in a fixed order into the npz layout, so
// the result is deterministic.  Every mbarrier wait is bounded; on timeout the
// roles raise the abort flag and the error flag, drain and free TMEM.
#include <algorithm>

#include <cuda.h>
#include <cuda_bf16.h>

#include "common.h"
#include "kernels.h"
#include "tc_util.cuh"

namespace cnncrf {
namespace k {

namespace {

constexpr int BM = 128;                  // output channels per tile (UMMA M)
constexpr int KT = 64;                   // pixels per K step
constexpr int BROWS = KT + 8;            // input pixels per step: the kx halo, whole 8-row swizzle atoms
constexpr int A_BOX = 64 * KT * 2;       // one 64-channel x 64-pixel dz box: 8 KB
constexpr int B_BOX = 64 * BROWS * 2;    // one 64-channel x 72-pixel input box: 9 KB
constexpr int A_BYTES = 2 * A_BOX;       // M = 128 channels: two boxes
constexpr int B_BYTES = 2 * B_BOX;       // N <= 128 channels: two boxes
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int NUM_THREADS = 192;
constexpr uint32_t TMEM_COLS = 512; // kw <= 3 accumulators of 128 columns
constexpr int MAX_STAGES = 6;
constexpr int SLACK = 16384; // shared memory past the barriers that no operand is placed in

struct WgTcParams {
    int n_img, Ho, Wo, chunks_x, kh, kw, np, cout, cin, a_boxes, b_boxes, stages;
    long steps, steps_per_split;
    float *part; // [split][ky][kx][cout][cin]
    int *err;
};

// One stage's MMAs, fully unrolled: KW taps x 4 K-steps of 16 pixels.  The
// descriptors advance by constants in their 16-byte start-address field: +128
// per K-step (16 rows of 128 B), +8 per tap (the input window starts one
// 128-byte row later).
template <int KW>
__device__ __forceinline__ void issue_stage(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, bool first)
{
#pragma unroll
    for (int kx = 0; kx < KW; ++kx)
#pragma unroll
        for (int kk = 0; kk < KT / 16; ++kk)
            tc::umma_bf16(tmem + kx * BM, da + 128 * kk, db + 8 * kx + 128 * kk, idesc, (first && kk == 0) ? 0u : 1u);
}

__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_wgrad_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const WgTcParams p)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = p.stages;
    uint64_t *full = (uint64_t *)(smem + S * STAGE_BYTES);
    uint64_t *empty = full + S;
    uint64_t *done = empty + S;
    uint64_t *drain = done + 1;
    uint32_t *tmem_slot = (uint32_t *)(drain + 1);
    volatile int *abort_flag = (volatile int *)(tmem_slot + 1);
    volatile int *zero_flag = abort_flag + 1;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ky = blockIdx.y, split = blockIdx.x;
    const long s0 = (long)split * p.steps_per_split, s1 = min(p.steps, s0 + p.steps_per_split);
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(done, 1);
        tc::mbar_init(drain, 1);
        *abort_flag = 0;
        *zero_flag = 0;
        tc::mbar_fence_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
    }
    if (warp == 1) {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    const long per_img = (long)p.Ho * p.chunks_x;

    if (warp == 0) {
        if (lane == 0) {
            int stage = 0, issued = 0;
            uint32_t phase = 0;
            bool ok = true;
            const uint32_t tx = (uint32_t)(p.a_boxes * A_BOX + p.b_boxes * B_BOX);
            for (long st = s0; st < s1 && ok; ++st) {
                const int img = (int)(st / per_img);
                const long r = st - (long)img * per_img;
                const int oy = (int)(r / p.chunks_x), x0 = (int)(r % p.chunks_x) * KT;
                if (!tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
                    ok = false;
                    break;
                }
                uint8_t *sa = smem + stage * STAGE_BYTES;
                tc::mbar_expect_tx(&full[stage], tx);
                for (int b = 0; b < p.a_boxes; ++b)
                    tc::tma_load_4d(sa + b * A_BOX, &tmA, &full[stage], b * 64, x0 + p.kw - 1, oy + p.kh - 1, img);
                for (int b = 0; b < p.b_boxes; ++b)
                    tc::tma_load_4d(sa + A_BYTES + b * B_BOX, &tmB, &full[stage], b * 64, x0, oy + ky, img);
                ++issued;
                if (++stage == S) {
                    stage = 0;
                    phase ^= 1;
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
            const uint32_t idesc = tc::idesc_bf16_mn(BM, p.np);
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (long st = s0; st < s1; ++st) {
                if (!tc::mbar_wait(&full[stage], phase, abort_flag)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t sa = tc::smem_u32(smem + stage * STAGE_BYTES);
                // a K step of 16 pixels = 16 rows of 128 bytes = two 8-row swizzle atoms; tap kx starts kx
                // rows into the input box (the swizzle follows the absolute address)
                const uint64_t da = tc::sdesc_sw128_mn(sa, A_BOX), db = tc::sdesc_sw128_mn(sa + A_BYTES, B_BOX);
                const bool first = st == s0;
                if (p.kw == 3) issue_stage<3>(tmem, da, db, idesc, first);
                else if (p.kw == 2) issue_stage<2>(tmem, da, db, idesc, first);
                else issue_stage<1>(tmem, da, db, idesc, first);
                tc::umma_commit(&empty[stage]);
                if (++stage == S) {
                    stage = 0;
                    phase ^= 1;
                }
            }
            if (ok) {
                tc::umma_commit(done);
            } else {
                *abort_flag = 1;
                atomicExch(p.err, 1);
            }
            // every MMA of this thread completes before TMEM is released
            tc::umma_commit(drain);
            tc::mbar_wait(drain, 0, zero_flag, 1u << 22);
        }
    } else {
        const int q = warp & 3, co = q * 32 + lane; // the TMEM lane quarter this warp may read
        int ok = 1;
        if (lane == 0) ok = tc::mbar_wait(done, 0, abort_flag) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        if (!ok) {
            *abort_flag = 1;
            atomicExch(p.err, 1);
        } else {
            tc::fence_after_sync();
            for (int kx = 0; kx < p.kw; ++kx) {
                float *dst = p.part + ((((long)split * p.kh + ky) * p.kw + kx) * p.cout + co) * p.cin;
                for (int c = 0; c < p.np / 16; ++c) {
                    float v[16];
                    tc::tmem_ld16(tmem + ((uint32_t)(q * 32) << 16) + kx * BM + c * 16, v); // warp-collective
                    if (co < p.cout)
#pragma unroll
                        for (int j = 0; j < 16; ++j)
                            if (c * 16 + j < p.cin) dst[c * 16 + j] = v[j];
                }
            }
        }
    }
    __syncthreads();
    if (warp == 1) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, TMEM_COLS);
    }
}

// dw[co][ci][kh-1-ky][kw-1-kx] += sum over splits of part[split][ky][kx][co][ci]:
// 32 outputs per CTA (one per lane), warp w sums splits w, w + 8, ..., then
// the 8 warp sums in a fixed order (deterministic)
__global__ void __launch_bounds__(256) k_wgrad_tc_reduce(const float *__restrict__ part, int nsplit, int kh, int kw,
                                                         int Cout, int Cin, float *__restrict__ dw)
{
    __shared__ float s[8][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long per = (long)kh * kw * Cout * Cin, i = (long)blockIdx.x * 32 + lane;
    float acc = 0.0f;
    if (i < per)
        for (int sp = w; sp < nsplit; sp += 8) acc += part[(long)sp * per + i];
    s[w][lane] = acc;
    __syncthreads();
    if (w != 0 || i >= per) return;
    float t = s[0][lane];
#pragma unroll
    for (int j = 1; j < 8; ++j) t += s[j][lane];
    const int ci = (int)(i % Cin);
    const long r = i / Cin;
    const int co = (int)(r % Cout), tt = (int)(r / Cout), kx = tt % kw, ky = tt / kw;
    dw[(((long)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)] += t;
}

size_t smem_bytes(int stages) { return 1024 + (size_t)stages * STAGE_BYTES + (2 * stages + 2) * 8 + 16 + SLACK; }

} // namespace

bool wgrad_tc_supported(int Cout, int Cin, int kh, int kw)
{
    // N = Cin rounded to 16 must fit one accumulator's 128 TMEM columns
    return Cout >= 1 && Cout <= BM && Cin >= 1 && Cin <= 128 && kw >= 1 && kw <= 3 && kh >= 1 && kh <= 3;
}

int wgrad_tc_splits(int kh, long steps)
{
    int sms = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        sms = 148;
    return (int)std::max(1L, std::min((long)std::max(1, sms / kh), steps));
}

size_t wgrad_tc_scratch_bytes(int Cout, int Cin, int kh, int kw, int splits)
{
    return 4 * (size_t)splits * kh * kw * Cout * Cin;
}

int wgrad_tc(const void *dzpad, int Cout, int cpa, const void *in, long in_pix, long in_row, long in_img, int Cin,
             int kh, int kw, int nimg, int Ho, int Wo, void *scratch, size_t scratch_bytes, float *dw, int *err,
             cudaStream_t st)
{
    if (!wgrad_tc_supported(Cout, Cin, kh, kw)) return fail(CNNCRF_EUNSUPPORTED, "wgrad_tc: shape");
    if (cpa % 64 || cpa < Cout || in_pix % 64 || in_pix < Cin)
        return fail(CNNCRF_EINVAL, "wgrad_tc: channel strides %d / %ld must be multiples of 64", cpa, in_pix);
    if (((uintptr_t)dzpad & 15) || ((uintptr_t)in & 15) || in_row % in_pix || in_img % in_row)
        return fail(CNNCRF_EINVAL, "wgrad_tc: operand layout");
    const int Hin = Ho + kh - 1, Win = Wo + kw - 1, chunks_x = ceil_div(Wo, KT);
    if (in_row / in_pix < Win || in_img / in_row < Hin) return fail(CNNCRF_EINVAL, "wgrad_tc: input extent");
    const long steps = (long)nimg * Ho * chunks_x;
    const int splits = wgrad_tc_splits(kh, steps);
    if (scratch_bytes < wgrad_tc_scratch_bytes(Cout, Cin, kh, kw, splits))
        return fail(CNNCRF_EINVAL, "wgrad_tc: scratch too small");
    auto enc = tc::tensor_map_encoder();
    if (!enc) return fail(CNNCRF_ECUDA, "wgrad_tc: cuTensorMapEncodeTiled unavailable");
    const int np = (Cin + 15) & ~15;
    CUtensorMap ma, mb;
    {
        const int Hp = Ho + 2 * (kh - 1), Wp = Wo + 2 * (kw - 1);
        cuuint64_t g[4] = {(cuuint64_t)cpa, (cuuint64_t)Wp, (cuuint64_t)Hp, (cuuint64_t)nimg};
        cuuint64_t s[3] = {(cuuint64_t)cpa * 2, (cuuint64_t)Wp * cpa * 2, (cuuint64_t)Hp * Wp * cpa * 2};
        cuuint32_t box[4] = {64, KT, 1, 1}, e[4] = {1, 1, 1, 1};
        CUresult r = enc(&ma, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)dzpad, g, s, box, e,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "wgrad_tc: output-gradient tensor map (%d)", (int)r);
    }
    {
        // the layer's input extent exactly (the rows may be a window of a wider image): nothing past it is read
        cuuint64_t g[4] = {(cuuint64_t)in_pix, (cuuint64_t)Win, (cuuint64_t)Hin, (cuuint64_t)nimg};
        cuuint64_t s[3] = {(cuuint64_t)in_pix * 2, (cuuint64_t)in_row * 2, (cuuint64_t)in_img * 2};
        cuuint32_t box[4] = {64, BROWS, 1, 1}, e[4] = {1, 1, 1, 1};
        CUresult r = enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, (void *)in, g, s, box, e,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "wgrad_tc: input tensor map (%d)", (int)r);
    }
    WgTcParams p{};
    p.n_img = nimg, p.Ho = Ho, p.Wo = Wo, p.chunks_x = chunks_x, p.kh = kh, p.kw = kw, p.np = np;
    p.cout = Cout, p.cin = Cin;
    // M = 128 always reads two channel boxes of dz; the second is loaded only when Cout > 64 (the rows
    // it would fill are not stored).  N = np reads a second input box when np > 64.
    p.a_boxes = Cout > 64 ? 2 : 1;
    p.b_boxes = np > 64 ? 2 : 1;
    p.steps = steps;
    p.steps_per_split = (steps + splits - 1) / splits;
    p.part = (float *)scratch;
    p.err = err;
    int dev = 0, maxsm = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    p.stages = 0;
    for (int s = 2; s <= MAX_STAGES; ++s)
        if (smem_bytes(s) <= (size_t)maxsm) p.stages = s;
    if (!p.stages) return fail(CNNCRF_EUNSUPPORTED, "wgrad_tc: shared memory");
    const size_t smem = smem_bytes(p.stages);
    CNNCRF_CUDA(cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // every split has at least one step: splits <= steps and steps_per_split = ceil(steps / splits)
    const int used = (int)((steps + p.steps_per_split - 1) / p.steps_per_split);
    {
        CNNCRF_PROF("wgrad_tc", st);
        k_wgrad_tc<<<dim3(used, kh), NUM_THREADS, smem, st>>>(ma, mb, p);
        const long per = (long)kh * kw * Cout * Cin;
        k_wgrad_tc_reduce<<<ceil_div(per, 32), 256, 0, st>>>(p.part, used, kh, kw, Cout, Cin, dw);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
