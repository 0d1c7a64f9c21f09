// k_wgrad_tc.cu -- the weight gradient of a kh x kw convolution layer on the
// tcgen05 tensor cores (training step, BF16 mode): BF16 operands, FP32
// accumulation in TMEM.
//
//   dW'[co][ky][kx][ci] = sum over pixels p = (img, oy, ox) of
//                         dz[p][co] * x[img][oy + ky][ox + kx][ci]
//
// is a GEMM per tap with M = output channels, N = input channels and K = the
// pixels.  Both operands must be K-major (pixels contiguous), so they are
// first written as planar BF16 copies: dzP[img][co][oy][ox] and, once per kx,
// xP[kx][img][ci][y][ox] = x[img][y][ox + kx][ci] (the kx shift is baked into
// the copy: a TMA box must start on a 16-byte boundary in x, and a K-major
// operand cannot start mid-row).  A K step is 64 consecutive pixels of one
// output row: one 128-row box of dzP (rows past Cout arrive as zeros) and kw
// boxes of xP at row oy + ky (rows past Cin and pixels past Wo arrive as
// zeros, so they add nothing).
//
// One CTA per (ky, pixel split), 192 threads:
//   warp 0      TMA: per K step one dzP box and kw xP boxes into a ring of stages
//   warp 1      TMEM allocation + single-thread tcgen05.mma, M = 128, N = NP,
//               K = 16 x 4 per box, into kw accumulators of 128 columns
//   warps 2..5  epilogue: warp q reads TMEM lanes (output channels) 32q..32q+31
//               of every accumulator and writes the split's FP32 partials
// A reduction kernel adds the splits in order into the npz layout, so the
// result is deterministic.  Every mbarrier wait is bounded; on timeout the
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

constexpr int BM = 128;        // output channels per tile (UMMA M)
constexpr int KT = 64;         // pixels per K step (one 128-byte BF16 row)
constexpr int A_BYTES = BM * 128;
constexpr int NUM_THREADS = 192;
constexpr uint32_t TMEM_COLS = 512; // kw <= 3 accumulators of 128 columns
constexpr int MAX_STAGES = 4;

struct WgTcParams {
    int n_img, Ho, Wo, chunks_x, kh, kw, np, cout, cin, stages, stage_bytes, b_bytes;
    long steps, steps_per_split;
    float *part; // [split][ky][kx][cout][cin]
    int *err;
};

__device__ __forceinline__ float ldv(const float *p) { return *p; }
__device__ __forceinline__ float ldv(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

// out[(z * C + c) * H * pitch + y * pitch + x] = in[img][y][x + shift][c] for
// x < Wout, z = zoff + img; a 32 x 32 (pixel x channel) tile through shared memory
template <class T>
__global__ void k_to_planar(const T *__restrict__ in, long in_pix, long in_row, long in_img, int C, int H, int Wout,
                            int shift, int zoff, int pitch, __nv_bfloat16 *__restrict__ out)
{
    __shared__ float t[32][33];
    const int x0 = blockIdx.x * 32, y = blockIdx.y % H, img = blockIdx.y / H, c0 = blockIdx.z * 32;
    const int tx = threadIdx.x, ty = threadIdx.y; // 32 x 8
    for (int i = ty; i < 32; i += 8) {
        const int x = x0 + i, c = c0 + tx;
        t[i][tx] = (x < Wout && c < C) ? ldv(in + img * in_img + (long)y * in_row + (long)(x + shift) * in_pix + c)
                                       : 0.0f;
    }
    __syncthreads();
    for (int i = ty; i < 32; i += 8) {
        const int c = c0 + i, x = x0 + tx;
        if (c < C && x < Wout)
            out[(((long)(zoff + img) * C + c) * H + y) * pitch + x] = __float2bfloat16_rn(t[tx][i]);
    }
}

__global__ void __launch_bounds__(NUM_THREADS, 1)
    k_wgrad_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const WgTcParams p)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = p.stages;
    uint64_t *full = (uint64_t *)(smem + S * p.stage_bytes);
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
            for (long st = s0; st < s1 && ok; ++st) {
                const int img = (int)(st / per_img);
                const long r = st - (long)img * per_img;
                const int oy = (int)(r / p.chunks_x), x0 = (int)(r % p.chunks_x) * KT;
                if (!tc::mbar_wait(&empty[stage], phase ^ 1, abort_flag)) {
                    ok = false;
                    break;
                }
                uint8_t *sa = smem + stage * p.stage_bytes;
                tc::mbar_expect_tx(&full[stage], p.stage_bytes);
                tc::tma_load_4d(sa, &tmA, &full[stage], x0, oy, 0, img);
                for (int kx = 0; kx < p.kw; ++kx)
                    tc::tma_load_4d(sa + A_BYTES + kx * p.b_bytes, &tmB, &full[stage], x0, oy + ky, 0,
                                    kx * p.n_img + img);
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
            const uint32_t idesc = tc::idesc_bf16(BM, p.np);
            int stage = 0;
            uint32_t phase = 0;
            bool ok = true;
            for (long st = s0; st < s1; ++st) {
                if (!tc::mbar_wait(&full[stage], phase, abort_flag)) {
                    ok = false;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t sa = tc::smem_u32(smem + stage * p.stage_bytes);
                const uint64_t da = tc::sdesc_sw128(sa);
                for (int kx = 0; kx < p.kw; ++kx) {
                    const uint64_t db = tc::sdesc_sw128(sa + A_BYTES + kx * p.b_bytes);
#pragma unroll
                    for (int kk = 0; kk < KT / 16; ++kk)
                        tc::umma_bf16(tmem + kx * BM, da + 2 * kk, db + 2 * kk, idesc, (st > s0 || kk > 0) ? 1u : 0u);
                }
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

// dw[co][ci][kh-1-ky][kw-1-kx] += sum over splits of part[split][ky][kx][co][ci], in split order
__global__ void k_wgrad_tc_reduce(const float *__restrict__ part, int nsplit, int kh, int kw, int Cout, int Cin,
                                  float *__restrict__ dw)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x, per = (long)kh * kw * Cout * Cin;
    if (i >= per) return;
    const int ci = (int)(i % Cin);
    const long r = i / Cin;
    const int co = (int)(r % Cout), t = (int)(r / Cout), kx = t % kw, ky = t / kw;
    float s = 0.0f;
    for (int sp = 0; sp < nsplit; ++sp) s += part[(long)sp * per + i];
    dw[(((long)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)] += s;
}

int planar_pitch(int W) { return (W + 7) & ~7; } // rows of 16-byte multiples, as TMA strides need

size_t smem_bytes(int stages, int stage_bytes) { return 1024 + (size_t)stages * stage_bytes + (2 * stages + 2) * 8 + 16; }

} // namespace

bool wgrad_tc_supported(int Cout, int Cin, int kh, int kw)
{
    // N = Cin rounded to 16 must fit one accumulator's 128 TMEM columns
    return Cout >= 1 && Cout <= BM && Cin >= 16 && Cin <= 128 && kw >= 1 && kw <= 3 && kh >= 1 && kh <= 3;
}

int wgrad_tc_splits(int kh, long steps)
{
    int sms = 0, dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        sms = 148;
    return (int)std::max(1L, std::min((long)std::max(1, sms / kh), steps));
}

size_t wgrad_tc_scratch_bytes(int nimg, int Ho, int Wo, int Hin, int Cout, int Cin, int kh, int kw, int splits)
{
    const size_t pitch = planar_pitch(Wo);
    const size_t a = 2 * (size_t)nimg * Cout * Ho * pitch, b = 2 * (size_t)kw * nimg * Cin * Hin * pitch;
    const size_t c = 4 * (size_t)splits * kh * kw * Cout * Cin;
    auto al = [](size_t x) { return (x + 1023) & ~(size_t)1023; };
    return al(a) + al(b) + al(c);
}

int wgrad_tc(const float *dz, int Cout, const void *in, long in_pix, long in_row, long in_img, int Cin, int kh,
             int kw, int nimg, int Ho, int Wo, void *scratch, size_t scratch_bytes, float *dw, int *err,
             cudaStream_t st)
{
    if (!wgrad_tc_supported(Cout, Cin, kh, kw)) return fail(CNNCRF_EUNSUPPORTED, "wgrad_tc: shape");
    const int Hin = Ho + kh - 1, chunks_x = ceil_div(Wo, KT), pitch = planar_pitch(Wo);
    const long steps = (long)nimg * Ho * chunks_x;
    const int splits = wgrad_tc_splits(kh, steps);
    if (scratch_bytes < wgrad_tc_scratch_bytes(nimg, Ho, Wo, Hin, Cout, Cin, kh, kw, splits))
        return fail(CNNCRF_EINVAL, "wgrad_tc: scratch too small");
    if (((uintptr_t)scratch & 1023) != 0) return fail(CNNCRF_EINVAL, "wgrad_tc: scratch not 1024-byte aligned");
    auto al = [](size_t x) { return (x + 1023) & ~(size_t)1023; };
    __nv_bfloat16 *dzP = (__nv_bfloat16 *)scratch;
    __nv_bfloat16 *xP = (__nv_bfloat16 *)((char *)scratch + al(2 * (size_t)nimg * Cout * Ho * pitch));
    float *part = (float *)((char *)xP + al(2 * (size_t)kw * nimg * Cin * Hin * pitch));
    {
        CNNCRF_PROF("wgrad_planar", st);
        k_to_planar<float><<<dim3(ceil_div(Wo, 32), Ho * nimg, ceil_div(Cout, 32)), dim3(32, 8), 0, st>>>(
            dz, Cout, (long)Wo * Cout, (long)Ho * Wo * Cout, Cout, Ho, Wo, 0, 0, pitch, dzP);
        for (int kx = 0; kx < kw; ++kx)
            k_to_planar<__nv_bfloat16><<<dim3(ceil_div(Wo, 32), Hin * nimg, ceil_div(Cin, 32)), dim3(32, 8), 0, st>>>(
                (const __nv_bfloat16 *)in, in_pix, in_row, in_img, Cin, Hin, Wo, kx, kx * nimg, pitch, xP);
    }
    auto enc = tc::tensor_map_encoder();
    if (!enc) return fail(CNNCRF_ECUDA, "wgrad_tc: cuTensorMapEncodeTiled unavailable");
    const int np = (Cin + 15) & ~15;
    CUtensorMap ma, mb;
    {
        cuuint64_t g[4] = {(cuuint64_t)Wo, (cuuint64_t)Ho, (cuuint64_t)Cout, (cuuint64_t)nimg};
        cuuint64_t s[3] = {(cuuint64_t)pitch * 2, (cuuint64_t)Ho * pitch * 2, (cuuint64_t)Cout * Ho * pitch * 2};
        cuuint32_t box[4] = {KT, 1, BM, 1}, e[4] = {1, 1, 1, 1};
        CUresult r = enc(&ma, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, dzP, g, s, box, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "wgrad_tc: output-gradient tensor map (%d)", (int)r);
    }
    {
        cuuint64_t g[4] = {(cuuint64_t)Wo, (cuuint64_t)Hin, (cuuint64_t)Cin, (cuuint64_t)kw * nimg};
        cuuint64_t s[3] = {(cuuint64_t)pitch * 2, (cuuint64_t)Hin * pitch * 2, (cuuint64_t)Cin * Hin * pitch * 2};
        cuuint32_t box[4] = {KT, 1, (cuuint32_t)np, 1}, e[4] = {1, 1, 1, 1};
        CUresult r = enc(&mb, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, xP, g, s, box, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(CNNCRF_ECUDA, "wgrad_tc: input tensor map (%d)", (int)r);
    }
    WgTcParams p{};
    p.n_img = nimg, p.Ho = Ho, p.Wo = Wo, p.chunks_x = chunks_x, p.kh = kh, p.kw = kw, p.np = np;
    p.cout = Cout, p.cin = Cin;
    p.b_bytes = np * 128; // np rows of 128 bytes: whole 1024-byte swizzle atoms, np being a multiple of 16
    p.stage_bytes = A_BYTES + kw * p.b_bytes;
    p.steps = steps;
    p.steps_per_split = (steps + splits - 1) / splits;
    p.part = part;
    p.err = err;
    int dev = 0, maxsm = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    p.stages = 0;
    for (int s = 2; s <= MAX_STAGES; ++s)
        if (smem_bytes(s, p.stage_bytes) <= (size_t)maxsm) p.stages = s;
    if (!p.stages) return fail(CNNCRF_EUNSUPPORTED, "wgrad_tc: shared memory");
    const size_t smem = smem_bytes(p.stages, p.stage_bytes);
    CNNCRF_CUDA(cudaFuncSetAttribute(k_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // every split has at least one step: splits <= steps and steps_per_split = ceil(steps / splits)
    const int used = (int)((steps + p.steps_per_split - 1) / p.steps_per_split);
    {
        CNNCRF_PROF("wgrad_tc", st);
        k_wgrad_tc<<<dim3(used, kh), NUM_THREADS, smem, st>>>(ma, mb, p);
        const long per = (long)kh * kw * Cout * Cin;
        k_wgrad_tc_reduce<<<ceil_div(per, 256), 256, 0, st>>>(part, used, kh, kw, Cout, Cin, dw);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
