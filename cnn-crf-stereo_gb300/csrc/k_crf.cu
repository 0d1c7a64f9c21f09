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
// warp shuffles, the minimum over labels from one redux.sync.min.f32.  All
// operations are exact (min) or single IEEE ops in the oracle's order, so the
// labels equal the oracle's bit for bit.  Compiled with --fmad=false.
#include <algorithm>
#include <vector>

#include "k_crf_chain.cuh"

namespace cnncrf {
namespace k {

int crf_pass_ring8(const CrfPassArgs &a, bool hpass, int delta, int wpb, cudaStream_t st)
{
    return launch_pass_any<8>(a, hpass, delta, wpb, st);
}

size_t crf_pass_smem(int P, int RING, int W, int H, bool hpass, int wpb)
{
    (void)W, (void)H; // the chains' weights stream through registers: no per-node shared memory
    return sizeof(float) * wpb * (size_t)ring_floats(P, RING, hpass);
}

namespace {

// One warp per pair: the bound = (sum of the H chain minima) + (sum of the V
// chain minima), each sum taken as 32 lane-strided FP64 partial sums (lane l
// over chains l, l + 32, .. in ascending order) added in lane order, so the
// dependent FP64 adds are about n / 32 + 31 instead of n (GB300's FP64 adds
// are slow).  The oracle sums in the same order.
__device__ __forceinline__ double sum32(const double *__restrict__ c, int n, int lane)
{
    double s = 0.0;
    for (int i = lane; i < n; i += 32) s += c[i];
    double t = __shfl_sync(0xffffffffu, s, 0);
#pragma unroll 1
    for (int l = 1; l < 32; ++l) t += __shfl_sync(0xffffffffu, s, l);
    return t;
}

__global__ void k_lb(const double *__restrict__ cH, int H, const double *__restrict__ cV, int W,
                     double *__restrict__ lb, int npairs)
{
    const int p = blockIdx.x, lane = threadIdx.x;
    if (p >= npairs) return;
    const double sh = sum32(cH + (long)p * H, H, lane), sv = sum32(cV + (long)p * W, W, lane);
    if (lane == 0) lb[p] = sh + sv;
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

__global__ void k_c1(const float *__restrict__ cost, const uint16_t *__restrict__ costq, float qs, float qo,
                     const float *__restrict__ phi, long n, float *__restrict__ out)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __fsub_rn(costq ? __fmaf_rn((float)costq[i], qs, qo) : cost[i], phi[i]);
}

struct Layout {
    size_t phi, lbuf, ch, cv, lb, total;
};

Layout layout(int W, int H, int D, int np = 1)
{
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    Layout l;
    size_t n = (size_t)W * H * D * np;
    l.phi = 0;
    l.lbuf = al(l.phi + n * sizeof(float));
    l.ch = al(l.lbuf + n * sizeof(float));
    l.cv = al(l.ch + (size_t)H * np * sizeof(double));
    l.lb = al(l.cv + (size_t)W * np * sizeof(double));
    l.total = al(l.lb + np * sizeof(double));
    return l;
}

int pass(const CrfPassArgs &a, bool hpass, int delta, int ring, int wpb, cudaStream_t st)
{
    return ring == 4 ? crf_pass_ring4(a, hpass, delta, wpb, st) : crf_pass_ring8(a, hpass, delta, wpb, st);
}

// labels per lane of the instantiated kernel (launch_pass_any's choice)
int lane_labels(int D)
{
    const int P = (D + 31) / 32;
    return P <= 4 ? P : (P <= 6 ? 6 : 8);
}

bool fits(int D, int W, int H, bool hpass, int ring, int wpb)
{
    return crf_pass_smem(lane_labels(D), ring, W, H, hpass, wpb) <= 227 * 1024;
}

// the tile of the tuning table for this shape, each pass falling back to the
// default when the tuned one does not fit the shared memory
CrfTile effective_tile(int W, int H, int D, int np, int delta)
{
    CrfTile t = crf_tile_lookup(W, H, D, np, delta), d;
    if (!fits(D, W, H, true, t.ring_h, t.wpb_h)) t.ring_h = d.ring_h, t.wpb_h = d.wpb_h;
    if (!fits(D, W, H, false, t.ring_v, t.wpb_v)) t.ring_v = d.ring_v, t.wpb_v = d.wpb_v;
    return t;
}

CrfPassArgs pass_args(const float *cost, long wps, int W, int H, int D, int np, const Rho &rp, char *ws,
                      const Layout &l, const void *costq, UnaryQ16 q)
{
    CrfPassArgs a{};
    a.theta = cost;
    a.thetaq = crf_reads_q16(D) ? (const uint16_t *)costq : nullptr;
    a.qscale = q.scale, a.qoffset = q.offset;
    // the kernels' dequantisation folds 2^23 scale into the offset (exact:
    // unary_q16 only hands out codes for which it is)
    a.qoffset23 = q.offset - 8388608.0f * q.scale;
    a.phi = (float *)(ws + l.phi);
    a.lbuf = (float *)(ws + l.lbuf);
    a.W = W, a.H = H, a.D = D, a.np = np, a.wps = wps;
    a.rp = rp;
    a.store_phi = 1;
    return a;
}

// keep_phi = false: the last V pass does not write phi (nothing reads C1 from this workspace afterwards)
int run_passes(const float *cost, const float *wx, const float *wy, long wps, int W, int H, int D, int np,
               const Rho &rp, int delta, int iters, int32_t *labels, char *ws, const Layout &l, cudaStream_t st,
               bool keep_phi, const void *costq, UnaryQ16 q)
{
    if (delta < 1 || delta > 4) return fail(CNNCRF_EUNSUPPORTED, "crf: delta %d outside 1..4", delta);
    const CrfTile t = effective_tile(W, H, D, np, delta);
    if (!fits(D, W, H, true, t.ring_h, t.wpb_h) || !fits(D, W, H, false, t.ring_v, t.wpb_v))
        return fail(CNNCRF_EUNSUPPORTED, "crf: the chain ring of this tile exceeds shared memory");
    double *cH = (double *)(ws + l.ch), *cV = (double *)(ws + l.cv), *lb = (double *)(ws + l.lb);
    CrfPassArgs a = pass_args(cost, wps, W, H, D, np, rp, ws, l, costq, q);
    for (int it = 0; it < iters; ++it) {
        a.wgt = wx, a.first = it == 0, a.labels = nullptr, a.cmin = cH;
        CNNCRF_TRY(pass(a, true, delta, t.ring_h, t.wpb_h, st));
        a.wgt = wy, a.first = 0, a.labels = it == iters - 1 ? labels : nullptr, a.cmin = cV;
        a.store_phi = keep_phi || it != iters - 1;
        CNNCRF_TRY(pass(a, false, delta, t.ring_v, t.wpb_v, st));
    }
    {
        CNNCRF_PROF("lb", st);
        k_lb<<<np, 32, 0, st>>>(cH, H, cV, W, lb, np);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

Rho make_rho(const CrfParams &p)
{
    Rho rp;
    rp.L2 = p.L2;
    rp.slack = p.slack;
    rp.rho[0] = 0.0f;
    for (int t = 1; t <= 8; ++t) rp.rho[t] = p.shape == 0 ? fminf(p.L1, p.L2) : fminf(p.L1 * (float)t, p.L2);
    return rp;
}

int check_args(const float *cost, const float *wx, const float *wy, int W, int H, int D, int np, const CrfParams &p,
               const void *ws, size_t ws_bytes)
{
    if (W < 1 || H < 1 || D < 1 || D > 256 || np < 1) return fail(CNNCRF_EINVAL, "crf: bad size %dx%dx%d x%d", W, H, D, np);
    if (!cost || !wx || !wy || !ws) return fail(CNNCRF_EINVAL, "crf: null pointer");
    if (p.slack <= 0.0f || p.slack > 1.0f) return fail(CNNCRF_EINVAL, "crf: slack %g outside (0,1]", p.slack);
    const Layout l = layout(W, H, D, np);
    if (ws_bytes < l.total) return fail(CNNCRF_EINVAL, "crf: workspace %zu < %zu bytes", ws_bytes, l.total);
    if (((uintptr_t)ws & 255) != 0) return fail(CNNCRF_EINVAL, "crf: workspace not 256-byte aligned");
    if (((uintptr_t)cost & 15) != 0) return fail(CNNCRF_EINVAL, "crf: cost volume not 16-byte aligned");
    return CNNCRF_OK;
}

int solve_impl(const float *cost, const float *wx, const float *wy, long wps, int W, int H, int D, int np,
               const CrfParams &p, int iters, int32_t *labels, void *ws, size_t ws_bytes, cudaStream_t st,
               bool keep_phi, const void *costq, UnaryQ16 q)
{
    CNNCRF_TRY(check_args(cost, wx, wy, W, H, D, np, p, ws, ws_bytes));
    if (!labels) return fail(CNNCRF_EINVAL, "crf: null pointer");
    const Layout l = layout(W, H, D, np);
    char *w = (char *)ws;
    if (iters <= 0) {
        {
            CNNCRF_PROF("wta", st);
            k_wta<<<ceil_div((long)W * H * np, 256), 256, 0, st>>>(cost, (long)W * H * np, D, labels);
        }
        CNNCRF_CUDA(cudaMemsetAsync(w + l.lb, 0, sizeof(double) * np, st));
        CNNCRF_CHECK_LAUNCH();
        return CNNCRF_OK;
    }
    return run_passes(cost, wx, wy, wps, W, H, D, np, make_rho(p), p.delta, iters, labels, w, l, st, keep_phi,
                      costq, q);
}

// time one H and one V pass of every candidate tile (events on `st`, best of
// `reps`); the workspace's messages are overwritten, the next solve starts
// afresh (its first H pass does not read them)
int autotune_impl(const float *cost, const float *wx, const float *wy, long wps, int W, int H, int D, int np,
                  const CrfParams &p, void *ws, size_t ws_bytes, cudaStream_t st, CrfTile *best, float *ms_h,
                  float *ms_v, const void *costq, UnaryQ16 q)
{
    CNNCRF_TRY(check_args(cost, wx, wy, W, H, D, np, p, ws, ws_bytes));
    if (p.delta < 1 || p.delta > 4) return fail(CNNCRF_EUNSUPPORTED, "crf: delta %d outside 1..4", p.delta);
    const Layout l = layout(W, H, D, np);
    char *w = (char *)ws;
    CrfPassArgs a = pass_args(cost, wps, W, H, D, np, make_rho(p), w, l, costq, q);
    const int rings[2] = {8, 4}, wpbs[3] = {2, 1, 4}; // the default first: it wins ties
    const int reps = 3;
    struct Cand {
        int ring, wpb;
        bool h, v;
        cudaEvent_t e[3 * 3];
    };
    std::vector<Cand> cands;
    for (int r : rings)
        for (int b : wpbs) {
            Cand c{r, b, fits(D, W, H, true, r, b), fits(D, W, H, false, r, b), {}};
            if (c.h || c.v) cands.push_back(c);
        }
    int rc = CNNCRF_OK;
    for (auto &c : cands)
        for (auto &e : c.e)
            if (rc == CNNCRF_OK && cudaEventCreate(&e) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "crf tune: event");
    for (int rep = 0; rep < reps && rc == CNNCRF_OK; ++rep)
        for (auto &c : cands) {
            cudaEvent_t *e = c.e + 3 * rep;
            if (cudaEventRecord(e[0], st) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "crf tune: record");
            a.wgt = wx, a.first = 1, a.labels = nullptr, a.cmin = (double *)(w + l.ch);
            if (rc == CNNCRF_OK && c.h) rc = pass(a, true, p.delta, c.ring, c.wpb, st);
            if (rc == CNNCRF_OK && cudaEventRecord(e[1], st) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "crf tune: record");
            a.wgt = wy, a.first = 0, a.cmin = (double *)(w + l.cv);
            if (rc == CNNCRF_OK && c.v) rc = pass(a, false, p.delta, c.ring, c.wpb, st);
            if (rc == CNNCRF_OK && cudaEventRecord(e[2], st) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "crf tune: record");
            if (rc != CNNCRF_OK) break;
        }
    if (rc == CNNCRF_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = fail(CNNCRF_ECUDA, "crf tune: sync");
    CrfTile t;
    float bh = 1e30f, bv = 1e30f;
    for (auto &c : cands) {
        float mh = 1e30f, mv = 1e30f;
        for (int rep = 0; rep < reps && rc == CNNCRF_OK; ++rep) {
            float x = 0, y = 0;
            cudaEventElapsedTime(&x, c.e[3 * rep], c.e[3 * rep + 1]);
            cudaEventElapsedTime(&y, c.e[3 * rep + 1], c.e[3 * rep + 2]);
            mh = std::min(mh, x), mv = std::min(mv, y);
        }
        if (c.h && mh < bh) bh = mh, t.ring_h = c.ring, t.wpb_h = c.wpb;
        if (c.v && mv < bv) bv = mv, t.ring_v = c.ring, t.wpb_v = c.wpb;
    }
    for (auto &c : cands)
        for (auto &e : c.e)
            if (e) cudaEventDestroy(e);
    if (rc != CNNCRF_OK) return rc;
    if (bh >= 1e30f || bv >= 1e30f) return fail(CNNCRF_EUNSUPPORTED, "crf tune: no tile fits %dx%dx%d", W, H, D);
    *best = t;
    if (ms_h) *ms_h = bh;
    if (ms_v) *ms_v = bv;
    return CNNCRF_OK;
}

} // namespace

size_t crf_workspace_bytes(int W, int H, int D, int npairs) { return layout(W, H, D, npairs).total; }

bool crf_reads_q16(int D)
{
    const int P = lane_labels(D);
    return D == 32 * P && P % 2 == 0;
}

int crf_solve(const float *cost, const float *wx, const float *wy, int W, int H, int D, const CrfParams &p,
              int iters, int32_t *labels, void *ws, size_t ws_bytes, double *h_lb, cudaStream_t st,
              const void *costq, UnaryQ16 q)
{
    CNNCRF_TRY(solve_impl(cost, wx, wy, 0, W, H, D, 1, p, iters, labels, ws, ws_bytes, st, true, costq, q));
    if (h_lb) {
        Layout l = layout(W, H, D, 1);
        CNNCRF_CUDA(cudaMemcpyAsync(h_lb, (char *)ws + l.lb, sizeof(double), cudaMemcpyDeviceToHost, st));
        CNNCRF_CUDA(cudaStreamSynchronize(st));
    }
    return CNNCRF_OK;
}

int crf_solve_batch(const float *cost, const float *pw, int W, int H, int D, int npairs, const CrfParams &p,
                    int iters, int32_t *labels, void *ws, size_t ws_bytes, cudaStream_t st, bool keep_phi,
                    const void *costq, UnaryQ16 q)
{
    const long N = (long)W * H;
    return solve_impl(cost, pw, pw + N, 2 * N, W, H, D, npairs, p, iters, labels, ws, ws_bytes, st, keep_phi,
                      costq, q);
}

int crf_autotune(const float *cost, const float *wx, const float *wy, long wps, int W, int H, int D, int npairs,
                 const CrfParams &p, void *ws, size_t ws_bytes, cudaStream_t st, bool store, const void *costq,
                 UnaryQ16 q)
{
    CrfTile t;
    float mh = 0, mv = 0;
    CNNCRF_TRY(autotune_impl(cost, wx, wy, wps, W, H, D, npairs, p, ws, ws_bytes, st, &t, &mh, &mv, costq, q));
    if (store) crf_tile_store(W, H, D, npairs, p.delta, t, mh, mv);
    return CNNCRF_OK;
}

const double *crf_lb_device(const void *ws, int W, int H, int D, int npairs)
{
    return (const double *)((const char *)ws + layout(W, H, D, npairs).lb);
}

int crf_c1(const float *cost, const void *ws, long n, float *out, cudaStream_t st, int D, const void *costq,
           UnaryQ16 q)
{
    const float *phi = (const float *)ws;
    const uint16_t *cq = (costq && crf_reads_q16(D)) ? (const uint16_t *)costq : nullptr;
    {
        CNNCRF_PROF("c1", st);
        k_c1<<<ceil_div(n, 256), 256, 0, st>>>(cost, cq, q.scale, q.offset, phi, n, out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
