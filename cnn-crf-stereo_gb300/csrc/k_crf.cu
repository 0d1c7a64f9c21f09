// k_crf.cu -- the 4-connected CRF MAP solve (our SlackProp restatement).
//
// The reference calls slack_prop_2D_alg (stereo/stereo.cpp:140-154), an
// un-vendored dependency (dependencies/slackprop is empty).  This file
// implements the solver spec written out in the CPU oracle (oracle_crf):
// dual decomposition of the grid into horizontal chains (H) and vertical
// chains (V) with unaries theta - phi and phi.  One iteration = an H pass and
// a V pass.  A pass runs, per chain, the min-sum forward messages and then a
// backward sweep that at each node forms the min-marginal m, hands the
// fraction `slack` of its excess m - min(m) to the other subproblem, and
// propagates the reduced unary backwards.  The chain minimum is preserved, so
// the FP64 bound (sum of chain minima) never decreases.  Labels = first
// argmin of the V min-marginals of the last iteration.
//
// Pairwise: w * rho(|t|), rho(0) = 0, rho(1..delta) per shape, L2 beyond; the
// min-convolution is out_k = min(v_k, v_{k+-t} + w rho_t, min(v) + w L2) - min(v).
//
// GPU layout: one warp per chain (a row for H, a column for V); lane j holds
// labels k = j*P .. j*P+P-1 in registers; neighbours across lanes come from
// warp shuffles, the minimum over labels from an xor-shuffle butterfly.  All
// operations are exact (min) or single IEEE ops in the oracle's order, so the
// labels equal the oracle's bit for bit.  Compiled with --fmad=false.
#include <cfloat>
#include <math_constants.h>

#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

struct Rho {
    float rho[9];
    float L2;
    float slack;
};

#define INF CUDART_INF_F

template <int P> __device__ __forceinline__ float warp_min(const float (&v)[P])
{
    float m = v[0];
#pragma unroll
    for (int r = 1; r < P; ++r) m = fminf(m, v[r]);
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) m = fminf(m, __shfl_xor_sync(0xffffffffu, m, off));
    return m;
}

template <int P> __device__ __forceinline__ void load_vec(const float *p, int lane, int D, float (&v)[P])
{
    const int k0 = lane * P;
    if (D == 32 * P && (P == 1 || P == 2 || P == 4 || P == 8)) {
        if constexpr (P == 1) {
            v[0] = p[k0];
        } else if constexpr (P == 2) {
            float2 t = *(const float2 *)(p + k0);
            v[0] = t.x, v[1] = t.y;
        } else if constexpr (P == 4) {
            float4 t = *(const float4 *)(p + k0);
            v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w;
        } else if constexpr (P == 8) {
            float4 t = *(const float4 *)(p + k0), u = *(const float4 *)(p + k0 + 4);
            v[0] = t.x, v[1] = t.y, v[2] = t.z, v[3] = t.w, v[4] = u.x, v[5] = u.y, v[6] = u.z, v[7] = u.w;
        }
        return;
    }
#pragma unroll
    for (int r = 0; r < P; ++r) v[r] = (k0 + r < D) ? p[k0 + r] : 0.0f;
}

template <int P> __device__ __forceinline__ void store_vec(float *p, int lane, int D, const float (&v)[P])
{
    const int k0 = lane * P;
    if (D == 32 * P && (P == 1 || P == 2 || P == 4 || P == 8)) {
        if constexpr (P == 1) {
            p[k0] = v[0];
        } else if constexpr (P == 2) {
            *(float2 *)(p + k0) = make_float2(v[0], v[1]);
        } else if constexpr (P == 4) {
            *(float4 *)(p + k0) = make_float4(v[0], v[1], v[2], v[3]);
        } else if constexpr (P == 8) {
            *(float4 *)(p + k0) = make_float4(v[0], v[1], v[2], v[3]);
            *(float4 *)(p + k0 + 4) = make_float4(v[4], v[5], v[6], v[7]);
        }
        return;
    }
#pragma unroll
    for (int r = 0; r < P; ++r)
        if (k0 + r < D) p[k0 + r] = v[r];
}

// out = minconv(v) - g, pads (k >= D) kept at +inf.
template <int P, int DELTA>
__device__ __forceinline__ void minconv(const float (&v)[P], float g, float w, const Rho &rp, int lane,
                                        int D, float (&out)[P])
{
    float c[DELTA + 1];
#pragma unroll
    for (int t = 1; t <= DELTA; ++t) c[t] = __fmul_rn(w, rp.rho[t]);
    const float base = __fadd_rn(g, __fmul_rn(w, rp.L2));
    // E[DELTA + i] = value at label lane*P + i, i in [-DELTA, P + DELTA)
    float E[P + 2 * DELTA];
#pragma unroll
    for (int i = -DELTA; i < P + DELTA; ++i) {
        float val;
        if (i >= 0 && i < P) {
            val = v[i];
        } else if (i >= P) {
            val = __shfl_down_sync(0xffffffffu, v[i % P], i / P);
        } else {
            int off = (-i + P - 1) / P;
            int reg = ((i % P) + P) % P;
            val = __shfl_up_sync(0xffffffffu, v[reg], off);
        }
        int kk = lane * P + i;
        E[DELTA + i] = (kk >= 0 && kk < D) ? val : INF;
    }
#pragma unroll
    for (int r = 0; r < P; ++r) {
        float o = E[DELTA + r];
#pragma unroll
        for (int t = 1; t <= DELTA; ++t) {
            o = fminf(o, __fadd_rn(E[DELTA + r - t], c[t]));
            o = fminf(o, __fadd_rn(E[DELTA + r + t], c[t]));
        }
        o = fminf(o, base);
        out[r] = (lane * P + r < D) ? __fsub_rn(o, g) : INF;
    }
}

// Horizontal pass: one warp per row y, chain over x, weights wx[y][x] on the
// edge x -> x+1; unary theta - phi; the handed-over slack is added to phi.
template <int P, int DELTA>
__global__ void __launch_bounds__(64)
    k_crf_h(const float *__restrict__ theta, float *__restrict__ phi, const float *__restrict__ wx,
            float *__restrict__ Lbuf, int W, int H, int D, Rho rp, int first, double *__restrict__ cH)
{
    const int lane = threadIdx.x & 31;
    const int y = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (y >= H) return;
    const long row = (long)y * W;
    float L[P], v[P], th[P], ph[P];
#pragma unroll
    for (int r = 0; r < P; ++r) L[r] = 0.0f, ph[r] = 0.0f;
    double acc = 0.0, cmin = 0.0;
    for (int x = 0; x < W; ++x) {
        const long pix = row + x;
        load_vec<P>(theta + pix * D, lane, D, th);
        if (!first) load_vec<P>(phi + pix * D, lane, D, ph);
        store_vec<P>(Lbuf + pix * D, lane, D, L);
#pragma unroll
        for (int r = 0; r < P; ++r)
            v[r] = (lane * P + r < D) ? __fadd_rn(L[r], __fsub_rn(th[r], ph[r])) : INF;
        float g = warp_min<P>(v);
        if (x < W - 1) {
            acc += (double)g;
            minconv<P, DELTA>(v, g, wx[pix], rp, lane, D, L);
        } else {
            cmin = acc + (double)g;
        }
    }
    float R[P], Lx[P], m[P], A[P];
#pragma unroll
    for (int r = 0; r < P; ++r) R[r] = 0.0f;
    for (int x = W - 1; x >= 0; --x) {
        const long pix = row + x;
        load_vec<P>(theta + pix * D, lane, D, th);
        if (!first) {
            load_vec<P>(phi + pix * D, lane, D, ph);
        } else {
#pragma unroll
            for (int r = 0; r < P; ++r) ph[r] = 0.0f; // phi starts at zero
        }
        load_vec<P>(Lbuf + pix * D, lane, D, Lx);
#pragma unroll
        for (int r = 0; r < P; ++r) {
            A[r] = __fsub_rn(th[r], ph[r]);
            m[r] = (lane * P + r < D) ? __fadd_rn(__fadd_rn(Lx[r], A[r]), R[r]) : INF;
        }
        const float mu = warp_min<P>(m);
#pragma unroll
        for (int r = 0; r < P; ++r) {
            float h = __fmul_rn(rp.slack, __fsub_rn(m[r], mu));
            A[r] = __fsub_rn(A[r], h);
            ph[r] = __fadd_rn(ph[r], h);
        }
        store_vec<P>(phi + pix * D, lane, D, ph);
        if (x > 0) {
#pragma unroll
            for (int r = 0; r < P; ++r) v[r] = (lane * P + r < D) ? __fadd_rn(A[r], R[r]) : INF;
            float g = warp_min<P>(v);
            minconv<P, DELTA>(v, g, wx[pix - 1], rp, lane, D, R);
        }
    }
    if (lane == 0) cH[y] = cmin;
}

// Vertical pass: one warp per column x, chain over y, weights wy[y][x] on the
// edge y -> y+1; unary phi; the handed-over slack is subtracted from phi.
template <int P, int DELTA>
__global__ void __launch_bounds__(64)
    k_crf_v(float *__restrict__ phi, const float *__restrict__ wy, float *__restrict__ Lbuf, int W,
            int H, int D, Rho rp, int32_t *__restrict__ labels, double *__restrict__ cV)
{
    const int lane = threadIdx.x & 31;
    const int x = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (x >= W) return;
    float L[P], v[P], B[P];
#pragma unroll
    for (int r = 0; r < P; ++r) L[r] = 0.0f;
    double acc = 0.0, cmin = 0.0;
    for (int y = 0; y < H; ++y) {
        const long pix = (long)y * W + x;
        load_vec<P>(phi + pix * D, lane, D, B);
        store_vec<P>(Lbuf + pix * D, lane, D, L);
#pragma unroll
        for (int r = 0; r < P; ++r) v[r] = (lane * P + r < D) ? __fadd_rn(L[r], B[r]) : INF;
        float g = warp_min<P>(v);
        if (y < H - 1) {
            acc += (double)g;
            minconv<P, DELTA>(v, g, wy[pix], rp, lane, D, L);
        } else {
            cmin = acc + (double)g;
        }
    }
    float R[P], Lx[P], m[P];
#pragma unroll
    for (int r = 0; r < P; ++r) R[r] = 0.0f;
    for (int y = H - 1; y >= 0; --y) {
        const long pix = (long)y * W + x;
        load_vec<P>(phi + pix * D, lane, D, B);
        load_vec<P>(Lbuf + pix * D, lane, D, Lx);
#pragma unroll
        for (int r = 0; r < P; ++r)
            m[r] = (lane * P + r < D) ? __fadd_rn(__fadd_rn(Lx[r], B[r]), R[r]) : INF;
        const float mu = warp_min<P>(m);
        if (labels) {
            int best = 0x7fffffff;
#pragma unroll
            for (int r = P - 1; r >= 0; --r)
                if (m[r] == mu && lane * P + r < D) best = lane * P + r;
#pragma unroll
            for (int off = 16; off >= 1; off >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, off));
            if (lane == 0) labels[pix] = best;
        }
#pragma unroll
        for (int r = 0; r < P; ++r) B[r] = __fsub_rn(B[r], __fmul_rn(rp.slack, __fsub_rn(m[r], mu)));
        store_vec<P>(phi + pix * D, lane, D, B);
        if (y > 0) {
#pragma unroll
            for (int r = 0; r < P; ++r) v[r] = (lane * P + r < D) ? __fadd_rn(B[r], R[r]) : INF;
            float g = warp_min<P>(v);
            minconv<P, DELTA>(v, g, wy[pix - W], rp, lane, D, R);
        }
    }
    if (lane == 0) cV[x] = cmin;
}

__global__ void k_lb(const double *__restrict__ cH, int H, const double *__restrict__ cV, int W,
                     double *__restrict__ lb)
{
    double sh = 0.0, sv = 0.0;
    for (int y = 0; y < H; ++y) sh += cH[y];
    for (int x = 0; x < W; ++x) sv += cV[x];
    *lb = sh + sv;
}

__global__ void k_wta(const float *__restrict__ cost, long npx, int D, int32_t *__restrict__ labels)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npx) return;
    const float *c = cost + i * D;
    int best = 0;
    for (int k = 1; k < D; ++k)
        if (c[k] < c[best]) best = k;
    labels[i] = best;
}

__global__ void k_c1(const float *__restrict__ cost, const float *__restrict__ phi, long n,
                     float *__restrict__ out)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __fsub_rn(cost[i], phi[i]);
}

struct Layout {
    size_t phi, lbuf, ch, cv, lb, total;
};

Layout layout(int W, int H, int D)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    Layout l;
    size_t n = (size_t)W * H * D;
    l.phi = 0;
    l.lbuf = al(l.phi + n * sizeof(float));
    l.ch = al(l.lbuf + n * sizeof(float));
    l.cv = al(l.ch + (size_t)H * sizeof(double));
    l.lb = al(l.cv + (size_t)W * sizeof(double));
    l.total = al(l.lb + sizeof(double));
    return l;
}

template <int P, int DELTA>
int run_passes(const float *cost, const float *wx, const float *wy, int W, int H, int D, const Rho &rp,
               int iters, int32_t *labels, char *ws, const Layout &l, cudaStream_t st)
{
    float *phi = (float *)(ws + l.phi), *lbuf = (float *)(ws + l.lbuf);
    double *cH = (double *)(ws + l.ch), *cV = (double *)(ws + l.cv), *lb = (double *)(ws + l.lb);
    const int wpb = 2;
    for (int it = 0; it < iters; ++it) {
        {
            CNNCRF_PROF("crf_h", st);
            k_crf_h<P, DELTA><<<ceil_div(H, wpb), 32 * wpb, 0, st>>>(cost, phi, wx, lbuf, W, H, D, rp,
                                                                 it == 0, cH);
        }
        {
            CNNCRF_PROF("crf_v", st);
            k_crf_v<P, DELTA><<<ceil_div(W, wpb), 32 * wpb, 0, st>>>(
            phi, wy, lbuf, W, H, D, rp, it == iters - 1 ? labels : nullptr, cV);
        }
    }
    {
        CNNCRF_PROF("lb", st);
        k_lb<<<1, 1, 0, st>>>(cH, H, cV, W, lb);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

template <int P>
int dispatch_delta(int delta, const float *cost, const float *wx, const float *wy, int W, int H, int D,
                   const Rho &rp, int iters, int32_t *labels, char *ws, const Layout &l, cudaStream_t st)
{
    switch (delta) {
    case 1: return run_passes<P, 1>(cost, wx, wy, W, H, D, rp, iters, labels, ws, l, st);
    case 2: return run_passes<P, 2>(cost, wx, wy, W, H, D, rp, iters, labels, ws, l, st);
    case 3: return run_passes<P, 3>(cost, wx, wy, W, H, D, rp, iters, labels, ws, l, st);
    case 4: return run_passes<P, 4>(cost, wx, wy, W, H, D, rp, iters, labels, ws, l, st);
    default: return fail(CNNCRF_EUNSUPPORTED, "crf: delta %d outside 1..4", delta);
    }
}

} // namespace

size_t crf_workspace_bytes(int W, int H, int D) { return layout(W, H, D).total; }

int crf_solve(const float *cost, const float *wx, const float *wy, int W, int H, int D, const CrfParams &p,
              int iters, int32_t *labels, void *ws, size_t ws_bytes, double *h_lb, cudaStream_t st)
{
    if (W < 1 || H < 1 || D < 1 || D > 256) return fail(CNNCRF_EINVAL, "crf: bad size %dx%dx%d", W, H, D);
    if (!cost || !wx || !wy || !labels || !ws) return fail(CNNCRF_EINVAL, "crf: null pointer");
    if (p.slack <= 0.0f || p.slack > 1.0f) return fail(CNNCRF_EINVAL, "crf: slack %g outside (0,1]", p.slack);
    Layout l = layout(W, H, D);
    if (ws_bytes < l.total) return fail(CNNCRF_EINVAL, "crf: workspace %zu < %zu bytes", ws_bytes, l.total);
    if (((uintptr_t)ws & 255) != 0) return fail(CNNCRF_EINVAL, "crf: workspace not 256-byte aligned");
    if (((uintptr_t)cost & 15) != 0) return fail(CNNCRF_EINVAL, "crf: cost volume not 16-byte aligned");
    char *w = (char *)ws;
    if (iters <= 0) {
        {
            CNNCRF_PROF("wta", st);
            k_wta<<<ceil_div((long)W * H, 256), 256, 0, st>>>(cost, (long)W * H, D, labels);
        }
        CNNCRF_CUDA(cudaMemsetAsync(w + l.lb, 0, sizeof(double), st));
        CNNCRF_CHECK_LAUNCH();
    } else {
        Rho rp;
        rp.L2 = p.L2;
        rp.slack = p.slack;
        rp.rho[0] = 0.0f;
        for (int t = 1; t <= 8; ++t)
            rp.rho[t] = p.shape == 0 ? fminf(p.L1, p.L2) : fminf(p.L1 * (float)t, p.L2);
        int P = (D + 31) / 32;
        int rc;
        if (P <= 1) rc = dispatch_delta<1>(p.delta, cost, wx, wy, W, H, D, rp, iters, labels, w, l, st);
        else if (P <= 2) rc = dispatch_delta<2>(p.delta, cost, wx, wy, W, H, D, rp, iters, labels, w, l, st);
        else if (P <= 3) rc = dispatch_delta<3>(p.delta, cost, wx, wy, W, H, D, rp, iters, labels, w, l, st);
        else if (P <= 4) rc = dispatch_delta<4>(p.delta, cost, wx, wy, W, H, D, rp, iters, labels, w, l, st);
        else if (P <= 6) rc = dispatch_delta<6>(p.delta, cost, wx, wy, W, H, D, rp, iters, labels, w, l, st);
        else rc = dispatch_delta<8>(p.delta, cost, wx, wy, W, H, D, rp, iters, labels, w, l, st);
        if (rc != CNNCRF_OK) return rc;
    }
    if (h_lb) {
        CNNCRF_CUDA(cudaMemcpyAsync(h_lb, w + l.lb, sizeof(double), cudaMemcpyDeviceToHost, st));
        CNNCRF_CUDA(cudaStreamSynchronize(st));
    }
    return CNNCRF_OK;
}

int crf_c1(const float *cost, const void *ws, long n, float *out, cudaStream_t st)
{
    const float *phi = (const float *)ws;
    {
        CNNCRF_PROF("c1", st);
        k_c1<<<ceil_div(n, 256), 256, 0, st>>>(cost, phi, n, out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
