// k_tv.cu -- the TV/Huber primal-dual refinement (the inner loop of
// cuda::fuseTHuberQuadFit, stereo/stereo.cu:1141-1166) as one fused kernel.
//
// The reference runs every iteration as three full-image passes: a copy
// u_ = u, ttvqf_primal_kernel (stereo/stereo.cu:701-729) and
// thuberqf_dual_kernel (stereo/stereo.cu:773-796).  Here one launch runs K
// iterations on a 64 x 32 pixel tile held on chip: each thread keeps four
// pixels' u, the fit's per-pixel constants, the weights and p, q in registers, and the
// values that neighbours read -- p.x - q.x, p.y - q.y (the primal's
// divergence) and u_ (the dual's gradient) -- go through shared memory.  The
// primal at (x, y) reads (x-1, y) and (x, y-1); the dual reads (x+1, y) and
// (x, y+1), so a tile's edge corrupts one more ring of pixels per iteration:
// the tile overlaps its neighbours by a halo of K pixels on every side and
// writes only its interior (64 - 2K) x (32 - 2K) block.  Neighbour indices
// are clamped to the image exactly as the reference's clamp-addressed
// texture reads are, so tiles on the image border see the same values as the
// unfused kernels.
//
// Tiles read the state (u, p, q) of the previous launch and write a second
// copy (a workspace ping-pong), since a tile's halo belongs to other tiles.
// The per-element arithmetic is the reference kernels', operation for
// operation -- the fused multiply-adds their default compilation contracts
// are written out as __fmaf_rn, the rest is single IEEE operations -- and the
// per-pixel constants of the primal update are the same operations hoisted
// out of the iteration loop, so the results equal both the CPU oracle and the
// reference's own kernels bit for bit.  Compiled with --fmad=false.
#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

constexpr int TX = 64, TY = 32, NT = 512, RS = NT / TX, RPT = TY / RS; // 4 rows per thread, 8 rows apart
constexpr int KMAX = 8;                                         // iterations per launch

__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fmaxf(lo, fminf(v, hi)); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// prox_p with alpha = 0 (stereo/stereo.cu:752-757)
__device__ __forceinline__ float prox_p0(float v, float beta, float sigma, float w)
{
    if (fabsf(v) <= __fmul_rn(w, 0.0f)) return v;
    float m = fmaxf(0.0f, __fmaf_rn(-sigma, beta, fabsf(v)));
    float r = __fmul_rn(m, v > 0.0f ? 1.0f : -1.0f);
    return clampf(r, -w, w);
}

struct TvArgs {
    const float *u_in;
    const float2 *p_in, *q_in; // null: p = q = 0
    const float *u0;
    const float2 *qf;
    const float *wx, *wy;
    float *u_out;
    float2 *p_out, *q_out;
    float *ubar_out; // the last iteration's u_ (null: not written)
    int W, H, K;
    float tau, sigma, half, C, eps;
};

__global__ void __launch_bounds__(NT, 2) k_tv_fused(const TvArgs a)
{
    __shared__ float sX[TY][TX], sY[TY][TX], sU[TY][TX];
    const int W = a.W, H = a.H, K = a.K;
    const int c = threadIdx.x & (TX - 1), r0 = threadIdx.x / TX;
    const int ex = blockIdx.x * (TX - 2 * K) - K, ey = blockIdx.y * (TY - 2 * K) - K;
    const int gx = ex + c;
    const bool colin = gx >= 0 && gx < W;
    // left / right neighbour columns: clamped to the image, then to the tile
    // (a clamp to the tile only happens at the tile's edge, inside the halo)
    const int cm = clampi((gx > 0 ? gx - 1 : 0) - ex, 0, TX - 1);
    const int cp = clampi((gx + 1 < W ? gx + 1 : W - 1) - ex, 0, TX - 1);

    // per pixel: the state (u, u_, p, q) and the primal's per-pixel constants,
    // computed once per launch with the operations the reference applies per
    // iteration: inner = a - b u0, den = 1 + tau b, the box u0 -+ step / 2
    float u[RPT], ub[RPT], px[RPT], py[RPT], qx[RPT], qy[RPT];
    float inn[RPT], den[RPT], lo[RPT], hi[RPT], wxr[RPT], wyr[RPT];
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int r = r0 + RS * j, gy = ey + r;
        float uz = 0.0f, fa = 0.0f, fb = 0.0f;
        u[j] = wxr[j] = wyr[j] = px[j] = py[j] = qx[j] = qy[j] = ub[j] = 0.0f;
        if (colin && gy >= 0 && gy < H) {
            const long i = (long)gy * W + gx;
            u[j] = a.u_in[i];
            uz = a.u0[i];
            const float2 f = a.qf[i];
            fa = f.x, fb = f.y;
            wxr[j] = a.wx[i], wyr[j] = a.wy[i];
            if (a.p_in) {
                const float2 pp = a.p_in[i], qq = a.q_in[i];
                px[j] = pp.x, py[j] = pp.y, qx[j] = qq.x, qy[j] = qq.y;
            }
        }
        inn[j] = __fmaf_rn(-fb, uz, fa);
        den[j] = __fmaf_rn(a.tau, fb, 1.0f);
        lo[j] = __fsub_rn(uz, a.half);
        hi[j] = __fadd_rn(uz, a.half);
        sX[r][c] = __fsub_rn(px[j], qx[j]);
        sY[r][c] = __fsub_rn(py[j], qy[j]);
    }
    __syncthreads();

    for (int it = 0; it < K; ++it) {
        // ---- primal (ttvqf_primal_kernel); u_ = u at the iteration's start
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            const int r = r0 + RS * j, gy = ey + r;
            const int rm = clampi((gy > 0 ? gy - 1 : 0) - ey, 0, TY - 1);
            const float Px = __fsub_rn(px[j], qx[j]), Py = __fsub_rn(py[j], qy[j]);
            const float X = sX[r][cm], Y = sY[rm][c];
            const float div = __fsub_rn(__fadd_rn(__fsub_rn(Px, X), Py), Y);
            float un = __fmaf_rn(a.tau, div, u[j]);
            const float num = __fmaf_rn(-a.tau, inn[j], un);
            un = clampf(__fdiv_rn(num, den[j]), lo[j], hi[j]);
            ub[j] = __fsub_rn(__fmul_rn(2.0f, un), u[j]);
            u[j] = un;
            sU[r][c] = ub[j];
        }
        __syncthreads();
        // ---- dual (thuberqf_dual_kernel), Huber parameter eps
        const float dd = __fmaf_rn(a.sigma, a.eps, 1.0f);
#pragma unroll
        for (int j = 0; j < RPT; ++j) {
            const int r = r0 + RS * j, gy = ey + r;
            const int rp = clampi((gy + 1 < H ? gy + 1 : H - 1) - ey, 0, TY - 1);
            const float uc = ub[j];
            const float dx = __fsub_rn(sU[r][cp], uc);
            const float dy = __fsub_rn(sU[rp][c], uc);
            const float pnx = __fmaf_rn(a.sigma, dx, px[j]), pny = __fmaf_rn(a.sigma, dy, py[j]);
            const float qnx = __fmaf_rn(a.sigma, dx, qx[j]), qny = __fmaf_rn(a.sigma, dy, qy[j]);
            px[j] = clampf(__fdiv_rn(pnx, dd), -wxr[j], wxr[j]);
            py[j] = clampf(__fdiv_rn(pny, dd), -wyr[j], wyr[j]);
            qx[j] = prox_p0(qnx, a.C, a.sigma, wxr[j]);
            qy[j] = prox_p0(qny, a.C, a.sigma, wyr[j]);
            // the primals of this iteration read sX / sY before the barrier above
            sX[r][c] = __fsub_rn(px[j], qx[j]);
            sY[r][c] = __fsub_rn(py[j], qy[j]);
        }
        __syncthreads(); // every dual has read sU before the next primal rewrites it
    }

    // ---- the interior block, inside the image
    if (!colin || c < K || c >= TX - K) return;
#pragma unroll
    for (int j = 0; j < RPT; ++j) {
        const int r = r0 + RS * j, gy = ey + r;
        if (r < K || r >= TY - K || gy < 0 || gy >= H) continue;
        const long i = (long)gy * W + gx;
        a.u_out[i] = u[j];
        a.p_out[i] = make_float2(px[j], py[j]);
        a.q_out[i] = make_float2(qx[j], qy[j]);
        if (a.ubar_out) a.ubar_out[i] = ub[j];
    }
}

struct TvWs {
    size_t u, p, q, total;
};

TvWs tv_ws_layout(int W, int H)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t n = (size_t)W * H;
    TvWs l;
    l.u = 0;
    l.p = al(n * sizeof(float));
    l.q = al(l.p + 2 * n * sizeof(float));
    l.total = al(l.q + 2 * n * sizeof(float));
    return l;
}

} // namespace

size_t tv_workspace_bytes(int W, int H) { return tv_ws_layout(W, H).total; }

// `iters` iterations from (u, p, q), or from (u, 0, 0) when pq_zero; the
// state ends in (u, p, q) and the last iteration's u_ in u_.  Launches of at
// most KMAX iterations, alternating between the caller's state and the
// workspace so that the last launch writes the caller's buffers.
int tv_iterate(float *u, float *u_, const float *u0, const float *qf, float *p, float *q, const float *wx,
               const float *wy, int W, int H, float C, float eps, float step, int iters, void *ws,
               size_t ws_bytes, bool pq_zero, cudaStream_t st)
{
    if (W < 1 || H < 1) return fail(CNNCRF_EINVAL, "tv: bad size %dx%d", W, H);
    const size_t n = (size_t)W * H;
    if (iters <= 0) {
        if (pq_zero) {
            CNNCRF_CUDA(cudaMemsetAsync(p, 0, 2 * n * sizeof(float), st));
            CNNCRF_CUDA(cudaMemsetAsync(q, 0, 2 * n * sizeof(float), st));
        }
        return CNNCRF_OK;
    }
    const TvWs l = tv_ws_layout(W, H);
    if (!ws || ws_bytes < l.total) return fail(CNNCRF_EINVAL, "tv: workspace %zu < %zu bytes", ws_bytes, l.total);
    if (((uintptr_t)ws & 255) != 0) return fail(CNNCRF_EINVAL, "tv: workspace not 256-byte aligned");
    char *w = (char *)ws;
    float *wu = (float *)(w + l.u);
    float2 *wp = (float2 *)(w + l.p), *wq = (float2 *)(w + l.q);
    // launches of near-equal iteration counts, at most KMAX each (the halo,
    // and so the recomputed fringe, grows with the count)
    const int L = (iters + KMAX - 1) / KMAX;
    // state sets: 0 = the caller's buffers, 1 = the workspace; launch l
    // writes set (L-1-l) % 2, so the last one writes the caller's
    int in_set = (L % 2 == 1) ? 1 : 0;
    if (in_set == 1) { // the first launch writes the caller's set: read a copy
        CNNCRF_CUDA(cudaMemcpyAsync(wu, u, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
        if (!pq_zero) {
            CNNCRF_CUDA(cudaMemcpyAsync(wp, p, 2 * n * sizeof(float), cudaMemcpyDeviceToDevice, st));
            CNNCRF_CUDA(cudaMemcpyAsync(wq, q, 2 * n * sizeof(float), cudaMemcpyDeviceToDevice, st));
        }
    }
    const float Lc = (float)sqrt(8.0);
    TvArgs a{};
    a.u0 = u0, a.qf = (const float2 *)qf, a.wx = wx, a.wy = wy;
    a.W = W, a.H = H;
    a.tau = 1.0f / Lc, a.sigma = 1.0f / Lc, a.half = 0.5f * step, a.C = C, a.eps = eps;
    int done = 0;
    for (int li = 0; li < L; ++li) {
        const int K = (iters - done + (L - li) - 1) / (L - li);
        const int out_set = (L - 1 - li) % 2;
        a.K = K;
        a.u_in = in_set ? wu : u;
        a.p_in = (li == 0 && pq_zero) ? nullptr : (in_set ? wp : (const float2 *)p);
        a.q_in = (li == 0 && pq_zero) ? nullptr : (in_set ? wq : (const float2 *)q);
        a.u_out = out_set ? wu : u;
        a.p_out = out_set ? wp : (float2 *)p;
        a.q_out = out_set ? wq : (float2 *)q;
        a.ubar_out = li == L - 1 ? u_ : nullptr;
        const dim3 grid(ceil_div(W, TX - 2 * K), ceil_div(H, TY - 2 * K));
        {
            CNNCRF_PROF("tv", st);
            k_tv_fused<<<grid, NT, 0, st>>>(a);
        }
        CNNCRF_CHECK_LAUNCH();
        in_set = out_set;
        done += K;
    }
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
