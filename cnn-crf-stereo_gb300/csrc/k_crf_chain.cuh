// k_crf_chain.cuh -- the chain pass of the CRF solve (k_crf.cu), shared by
// the translation units that instantiate it for one prefetch depth each
// (k_crf.cu: 8 chain steps, k_crf_r4.cu: 4), so the variants the tile tuner
// chooses between compile in parallel.  Everything device-side has internal
// linkage; each unit exports one launcher, crf_pass_ring<RING>.
#ifndef CNNCRF_K_CRF_CHAIN_CUH
#define CNNCRF_K_CRF_CHAIN_CUH

#include <cfloat>
#include <math_constants.h>

#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

// pairwise term: rho[t] for |t| = 0..8 (t > delta: L2), slack fraction
struct Rho {
    float rho[9];
    float L2;
    float slack;
};

// one pass over all chains of one direction (see k_crf_chain)
struct CrfPassArgs {
    const float *theta; // the cost volume [np][H][W][D]
    const uint16_t *thetaq; // its 16-bit fixed-point copy, read by the H pass instead of theta when set
    float qscale, qoffset;  // theta = q * qscale + qoffset (exact in FP32)
    float qoffset23;        // qoffset - 2^23 qscale, exact: theta = (2^23 + q) * qscale + qoffset23
    float *phi;         // H/V split of the unary, same layout
    const float *wgt;   // wx (H pass) or wy (V pass), pair stride wps
    float *lbuf;        // forward messages, same layout as phi
    int W, H, D, np;
    long wps;
    Rho rp;
    int first;           // H pass of the first iteration: phi = 0, not read
    int store_phi;       // 0: the pass's phi is dead (the last V pass when no caller reads C1), not written
    int32_t *labels;     // V pass of the last iteration: argmin labels, else null
    double *cmin;        // per chain minimum [np][chains]
};

// launch one pass with prefetch depth RING (4 or 8) and `wpb` warps (chains)
// per CTA; EUNSUPPORTED when the CTA's shared memory would exceed the limit
int crf_pass_ring8(const CrfPassArgs &a, bool hpass, int delta, int wpb, cudaStream_t st);
int crf_pass_ring4(const CrfPassArgs &a, bool hpass, int delta, int wpb, cudaStream_t st);
size_t crf_pass_smem(int P, int RING, int W, int H, bool hpass, int wpb);

namespace {

#define INF CUDART_INF_F

// The warp minimum of the lanes' minima: one redux.sync.min.f32 (sm_100 and
// later), exact like a float min.  The chain values are never NaN (pads are
// +inf); a zero may come back with either sign, which no later operation
// distinguishes (the labels compare values, the bound adds them).
template <int P> __device__ __forceinline__ float warp_min(const float (&v)[P])
{
    float m = v[0];
#pragma unroll
    for (int r = 1; r < P; ++r) m = fminf(m, v[r]);
    float w;
    asm("redux.sync.min.f32 %0, %1, 0xffffffff;" : "=f"(w) : "f"(m));
    return w;
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

// Exact two-lane IEEE add (add.rn.f32x2) and three-input minimum (min.f32
// with three sources): the same values as two __fadd_rn and two fminf, in
// fewer instructions.
__device__ __forceinline__ void add2(float a0, float a1, float b, float &d0, float &d1)
{
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %4};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(d0), "=f"(d1)
        : "f"(a0), "f"(a1), "f"(b));
}
__device__ __forceinline__ float min3(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// out = minconv(v) - g, pads (k >= D) kept at +inf.  FULL: D == 32 * P (no
// pad labels, only the chain ends of lanes 0 and 31 are masked).
template <int P, int DELTA, bool FULL>
__device__ __forceinline__ void minconv(const float (&v)[P], float g, float w, const Rho &rp, int lane,
                                        int D, float (&out)[P])
{
    constexpr int NE = P + 2 * DELTA;       // labels lane*P - DELTA .. lane*P + P + DELTA - 1
    constexpr int NE2 = (NE + 1) / 2 * 2;   // padded to whole pairs
    float c[DELTA + 1];
#pragma unroll
    for (int t = 1; t <= DELTA; ++t) c[t] = __fmul_rn(w, rp.rho[t]);
    const float base = __fadd_rn(g, __fmul_rn(w, rp.L2));
    const int DD = FULL ? 32 * P : D;
    // E[DELTA + i] = value at label lane*P + i, i in [-DELTA, P + DELTA)
    float E[NE2];
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
        const int kk = lane * P + i;
        E[DELTA + i] = (kk >= 0 && kk < DD) ? val : INF;
    }
    if (NE2 > NE) E[NE2 - 1] = INF;
    float o[P];
#pragma unroll
    for (int r = 0; r < P; ++r) o[r] = E[DELTA + r];
#pragma unroll
    for (int t = 1; t <= DELTA; ++t) {
        float S[NE2]; // S[j] = E[j] + c[t]
#pragma unroll
        for (int q = 0; q < NE2; q += 2) add2(E[q], E[q + 1], c[t], S[q], S[q + 1]);
#pragma unroll
        for (int r = 0; r < P; ++r) o[r] = min3(o[r], S[DELTA + r - t], S[DELTA + r + t]);
    }
#pragma unroll
    for (int r = 0; r < P; ++r) out[r] = (FULL || lane * P + r < D) ? __fsub_rn(fminf(o[r], base), g) : INF;
}

// ---------------------------------------------------------------- cp.async ring
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(uint32_t dst, const void *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(uint32_t dst, const void *src, int bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// copy this lane's P labels of one pixel vector into its ring slot
template <int P> __device__ __forceinline__ void lane_copy(float *dst, const float *src, int lane, int D)
{
    const int k0 = lane * P;
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst + k0);
    if (D == 32 * P) {
        if constexpr (P % 4 == 0) {
#pragma unroll
            for (int i = 0; i < P / 4; ++i) cp_async16(d + 16 * i, src + k0 + 4 * i);
        } else if constexpr (P % 2 == 0) {
#pragma unroll
            for (int i = 0; i < P / 2; ++i) cp_async8(d + 8 * i, src + k0 + 2 * i);
        } else {
#pragma unroll
            for (int i = 0; i < P; ++i) cp_async4(d + 4 * i, src + k0 + i, 4);
        }
    } else {
#pragma unroll
        for (int i = 0; i < P; ++i) {
            const bool ok = k0 + i < D;
            cp_async4(d + 4 * i, ok ? src + k0 + i : src, ok ? 4 : 0);
        }
    }
}

// the same for a 16-bit unary vector: this lane's P values (2P bytes, P even:
// 4-byte aligned at any lane) into the first half of its slot
template <int P> __device__ __forceinline__ void lane_copy16(float *dst, const uint16_t *src, int lane)
{
    static_assert(P % 2 == 0, "16-bit theta copies need an even label count per lane");
    const int k0 = lane * P;
    const uint32_t d = (uint32_t)__cvta_generic_to_shared((uint16_t *)dst + k0);
    if constexpr (P % 8 == 0) {
#pragma unroll
        for (int i = 0; i < P / 8; ++i) cp_async16(d + 16 * i, src + k0 + 8 * i);
    } else if constexpr (P % 4 == 0) {
#pragma unroll
        for (int i = 0; i < P / 4; ++i) cp_async8(d + 8 * i, src + k0 + 4 * i);
    } else {
#pragma unroll
        for (int i = 0; i < P / 2; ++i) cp_async4(d + 4 * i, src + k0 + 2 * i, 4);
    }
}

// The whole warp copies one pixel vector of NB bytes (a multiple of 16, the
// source 16-byte aligned) into its ring slot in 16-byte chunks, lane l taking
// chunks l, l + 32, ..: one or two copy instructions per lane, with the
// chunk count known at compile time, where a lane copying its own labels
// takes up to three smaller copies and a run-time check of the label count.
// Other lanes' chunks are visible to a lane after its wait and a __syncwarp.
template <int NB> __device__ __forceinline__ void warp_copy(void *dst, const void *src, int lane)
{
    static_assert(NB % 16 == 0, "whole 16-byte chunks");
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
#pragma unroll
    for (int ch = 0; ch < (NB / 16 + 31) / 32; ++ch) {
        const int k = lane + 32 * ch;
        if (k < NB / 16) cp_async16(d + 16 * k, (const char *)src + 16 * k);
    }
}

// dequantise: q * scale + offset is exact (q < 2^16, scale a power of two,
// the sum a multiple of scale below 2^9 in magnitude).  The code goes into
// the low mantissa bits of 2^23 by one byte permute, which makes the float
// 2^23 + q exactly, and offset23 = offset - 2^23 scale (exact, checked on the
// host) takes the 2^23 back out inside the one rounding of the fma:
// (2^23 + q) scale + offset23 = q scale + offset.  Two instructions per label
// instead of a mask or shift, a conversion and the fma.
template <int P>
__device__ __forceinline__ void lane_read16(const float *slot, int lane, float scale, float offset23, float (&v)[P])
{
    const uint32_t *q = (const uint32_t *)((const uint16_t *)slot + lane * P);
#pragma unroll
    for (int i = 0; i < P / 2; ++i) {
        const uint32_t w = q[i];
        const float lo = __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7410)); // bytes w0, w1, 0x00, 0x4B
        const float hi = __int_as_float((int)__byte_perm(w, 0x4B000000u, 0x7432)); // bytes w2, w3, 0x00, 0x4B
        v[2 * i] = __fmaf_rn(lo, scale, offset23);
        v[2 * i + 1] = __fmaf_rn(hi, scale, offset23);
    }
}

template <int P> __device__ __forceinline__ void lane_read(const float *slot, int lane, float (&v)[P])
{
    const float *q = slot + lane * P; // 16-byte aligned for P % 4 == 0, 8-byte for P == 2
    if constexpr (P % 4 == 0) {
#pragma unroll
        for (int i = 0; i < P / 4; ++i) {
            const float4 t = *(const float4 *)(q + 4 * i);
            v[4 * i] = t.x, v[4 * i + 1] = t.y, v[4 * i + 2] = t.z, v[4 * i + 3] = t.w;
        }
    } else if constexpr (P == 2) {
        const float2 t = *(const float2 *)q;
        v[0] = t.x, v[1] = t.y;
    } else {
#pragma unroll
        for (int r = 0; r < P; ++r) v[r] = q[r];
    }
}

// floats of the ring per step: theta, phi and the forward message (H pass); phi and the message (V pass, no theta)
// (the theta slot holds 16-bit codes when t16: half the floats)
__host__ __device__ constexpr int theta_floats(int P, bool hpass, bool t16) { return hpass ? (t16 ? 16 * P : 32 * P) : 0; }
__host__ __device__ constexpr int ring_floats(int P, int RING, bool hpass, bool t16 = false)
{
    return RING * (theta_floats(P, hpass, t16) + 64 * P);
}

// One pass over the chains of one direction; one warp per chain.
//   HPASS: chain = row y over x (weights wx[y][x] on edge x -> x+1), unary
//          theta - phi, the handed-over slack is added to phi.
//   !HPASS: chain = column x over y (weights wy[y][x] on edge y -> y+1),
//          unary phi, the handed-over slack is subtracted from phi; labels
//          (if given) = first argmin of the min-marginals.
// Per step the pixel vectors come from a per-warp shared-memory ring filled
// RING steps ahead with cp.async (each lane copies and reads only its own
// labels), so the chain's dependent arithmetic does not wait on DRAM.
template <int P, int DELTA, bool HPASS, bool FULL, int RING, bool T16 = false, bool COOP = false>
__global__ void __launch_bounds__(128)
    k_crf_chain(const float *__restrict__ theta, const uint16_t *__restrict__ thetaq, float qscale, float qoffset23,
                float *__restrict__ phi, const float *__restrict__ wgt,
                float *__restrict__ Lbuf, int W, int H, int D, Rho rp, int first, int store_phi,
                int32_t *__restrict__ labels, double *__restrict__ cmin_out, int npairs, long wps)
{
    extern __shared__ float4 smem4[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gchain = blockIdx.x * (blockDim.x >> 5) + wib;
    const int n = HPASS ? W : H;
    const int nch = HPASS ? H : W;
    if (gchain >= nch * npairs) return;
    // pair of the batch and chain within it
    const int pair = gchain / nch, chain = gchain - pair * nch;
    const long pnd = (long)W * H * D * pair;
    theta += pnd;
    if (T16) thetaq += pnd;
    phi += pnd;
    Lbuf += pnd;
    wgt += wps * pair;
    if (labels) labels += (long)W * H * pair;
    cmin_out += (long)nch * pair;
    float *ring = (float *)smem4 + (size_t)wib * ring_floats(P, RING, HPASS, T16);
    auto pix = [&](int i) -> long { return HPASS ? (long)chain * W + i : (long)i * W + chain; };
    // Edge weights in registers: lane l holds the weight of edge 32 b + l of
    // the sweep's current block b (wc) and of the block it reaches next (wn),
    // one load per lane and block; a step's weight is a shuffle that depends
    // on no chain state, so shared memory does not grow with the chain.
    auto wload = [&](int b) -> float {
        const int e = 32 * b + lane;
        return (b >= 0 && e < n) ? __ldg(wgt + pix(e)) : 0.0f;
    };
    const bool use_phi = !(HPASS && first);
    // slot a of step i: 0 theta (H pass only), 1 phi, 2 the forward message
    constexpr int TF = theta_floats(P, HPASS, T16), SF = TF + 64 * P;
    auto slot = [&](int i, int a) { return ring + (i % RING) * SF + (a == 0 ? 0 : TF + (a - 1) * 32 * P); };

    // element offsets of the chain's nodes: node i at cb + i ns; the sweeps
    // step running offsets by ns instead of multiplying per node
    const long cb = pix(0) * D, ns = (HPASS ? 1L : (long)W) * D;

    // ---- forward: messages into each node, stored for the backward sweep
    // COOP (label counts that fill whole warps, 16-byte aligned vectors): the
    // warp copies each vector in 16-byte chunks instead of each lane its labels
    static_assert(!COOP || FULL, "cooperative copies: label counts that fill whole warps");
    auto issue_f = [&](int i, long o) { // node i, at element offset o
        if (i < n) {
            if constexpr (COOP) {
                if constexpr (HPASS && T16) warp_copy<64 * P>(slot(i, 0), thetaq + o, lane);
                else if (HPASS) warp_copy<128 * P>(slot(i, 0), theta + o, lane);
                if (use_phi) warp_copy<128 * P>(slot(i, 1), phi + o, lane);
            } else {
                if constexpr (HPASS && T16) lane_copy16<P>(slot(i, 0), thetaq + o, lane);
                else if (HPASS) lane_copy<P>(slot(i, 0), theta + o, lane, D);
                if (use_phi) lane_copy<P>(slot(i, 1), phi + o, lane, D);
            }
        }
        cp_commit();
    };
    float L[P], v[P], th[P], ph[P];
#pragma unroll
    for (int r = 0; r < P; ++r) L[r] = 0.0f, th[r] = 0.0f, ph[r] = 0.0f;
    long po = cb, so = cb; // the node being prefetched, the node being stored
    for (int i = 0; i < RING - 1; ++i, po += ns) issue_f(i, po);
    // the chain's minimum in FP64: lane l sums the node minima g_i of i = l mod 32
    // in ascending i, and the 32 partial sums are added in lane order at the end
    // of the sweep.  Within a block of 32 nodes lane l keeps node 32 b + l's
    // minimum as a float (gb) and adds it once, at the block's end: one FP64
    // conversion and add per 32 nodes, none on the message chain
    double acc = 0.0;
    float wn = wload(0);
    // blocks of 32 nodes: the block's weights in wc, the next block's loading into wn
    for (int b = 0, i = 0; i < n; ++b) {
    const float wc = wn;
    wn = wload(b + 1);
    const int iend = min(n, i + 32), nb = iend - i;
    float gb = 0.0f;
#pragma unroll (HPASS ? 1 : 2)
    for (; i < iend; ++i) {
        issue_f(i + RING - 1, po);
        po += ns;
        cp_wait<RING - 1>();
        if constexpr (COOP) __syncwarp(); // the other lanes' chunks of node i
        if constexpr (HPASS && T16) lane_read16<P>(slot(i, 0), lane, qscale, qoffset23, th);
        else if (HPASS) lane_read<P>(slot(i, 0), lane, th);
        if (use_phi) lane_read<P>(slot(i, 1), lane, ph);
        store_vec<P>(Lbuf + so, lane, D, L);
        so += ns;
#pragma unroll
        for (int r = 0; r < P; ++r) {
            const float un = HPASS ? __fsub_rn(th[r], ph[r]) : ph[r];
            v[r] = (FULL || lane * P + r < D) ? __fadd_rn(L[r], un) : INF;
        }
        const float g = warp_min<P>(v);
        gb = lane == (i & 31) ? g : gb;
        if (i < n - 1) minconv<P, DELTA, FULL>(v, g, __shfl_sync(0xffffffffu, wc, i & 31), rp, lane, D, L);
    }
    if (lane < nb) acc += (double)gb;
    }
    cp_wait<0>();
    double cmin = acc; // lane 0: ((p0 + p1) + p2) + ... + p31
#pragma unroll 1
    for (int l = 1; l < 32; ++l) {
        const double pl = __shfl_sync(0xffffffffu, acc, l);
        if (lane == 0) cmin += pl;
    }

    // ---- backward: min-marginals, slack hand-over, reduced unary propagated back
    auto issue_b = [&](int j, long o) { // j-th step of the sweep = node n-1-j, at element offset o
        if (j < n) {
            if constexpr (COOP) {
                if constexpr (HPASS && T16) warp_copy<64 * P>(slot(j, 0), thetaq + o, lane);
                else if (HPASS) warp_copy<128 * P>(slot(j, 0), theta + o, lane);
                if (use_phi) warp_copy<128 * P>(slot(j, 1), phi + o, lane);
                warp_copy<128 * P>(slot(j, 2), Lbuf + o, lane);
            } else {
                if constexpr (HPASS && T16) lane_copy16<P>(slot(j, 0), thetaq + o, lane);
                else if (HPASS) lane_copy<P>(slot(j, 0), theta + o, lane, D);
                if (use_phi) lane_copy<P>(slot(j, 1), phi + o, lane, D);
                lane_copy<P>(slot(j, 2), Lbuf + o, lane, D);
            }
        }
        cp_commit();
    };
    float R[P], Lx[P], m[P], A[P];
#pragma unroll
    for (int r = 0; r < P; ++r) R[r] = 0.0f;
    po = so = cb + (long)(n - 1) * ns;                 // both sweep down from node n-1
    long lpix = pix(n - 1);                            // the label's pixel (V pass)
    for (int j = 0; j < RING - 1; ++j, po -= ns) issue_b(j, po);
    // the sweep reads edges n-2 down to 0, in blocks of 32 edges from the top;
    // node 0 (no edge below it) comes last, in a block of its own
    wn = wload((n - 2) >> 5);
    for (int eb = (n - 2) >> 5, j = 0; j < n; --eb) {
    const float wc = wn;
    wn = wload(eb - 1);
    const int jend = eb >= 0 ? n - 1 - 32 * eb : n; // nodes i = e + 1 for the block's edges e
#pragma unroll (HPASS ? 1 : 2)
    for (; j < jend; ++j) {
        const int i = n - 1 - j, e = i - 1; // edge e -> i
        issue_b(j + RING - 1, po);
        po -= ns;
        cp_wait<RING - 1>();
        if constexpr (COOP) __syncwarp();
        if constexpr (HPASS && T16) lane_read16<P>(slot(j, 0), lane, qscale, qoffset23, th);
        else if (HPASS) lane_read<P>(slot(j, 0), lane, th);
        if (use_phi) {
            lane_read<P>(slot(j, 1), lane, ph);
        } else {
#pragma unroll
            for (int r = 0; r < P; ++r) ph[r] = 0.0f; // phi starts at zero
        }
        lane_read<P>(slot(j, 2), lane, Lx);
#pragma unroll
        for (int r = 0; r < P; ++r) {
            A[r] = HPASS ? __fsub_rn(th[r], ph[r]) : ph[r];
            m[r] = (FULL || lane * P + r < D) ? __fadd_rn(__fadd_rn(Lx[r], A[r]), R[r]) : INF;
        }
        const float mu = warp_min<P>(m);
        if (!HPASS && labels) {
            int best = 0x7fffffff;
#pragma unroll
            for (int r = P - 1; r >= 0; --r)
                if (m[r] == mu && (FULL || lane * P + r < D)) best = lane * P + r;
            best = __reduce_min_sync(0xffffffffu, best);
            if (lane == 0) labels[lpix] = best;
            lpix -= W;
        }
#pragma unroll
        for (int r = 0; r < P; ++r) {
            const float h = __fmul_rn(rp.slack, __fsub_rn(m[r], mu));
            A[r] = __fsub_rn(A[r], h);
            ph[r] = HPASS ? __fadd_rn(ph[r], h) : A[r];
        }
        if (store_phi) store_vec<P>(phi + so, lane, D, ph);
        so -= ns;
        if (i > 0) {
#pragma unroll
            for (int r = 0; r < P; ++r) v[r] = (FULL || lane * P + r < D) ? __fadd_rn(A[r], R[r]) : INF;
            const float g = warp_min<P>(v);
            minconv<P, DELTA, FULL>(v, g, __shfl_sync(0xffffffffu, wc, e & 31), rp, lane, D, R);
        }
    }
    }
    cp_wait<0>();
    if (lane == 0) cmin_out[chain] = cmin;
}

template <int P, int DELTA, int RING>
int launch_pass(const CrfPassArgs &a, bool hpass, int wpb, cudaStream_t st)
{
    const bool full = a.D == 32 * P;
    // the H pass on the 16-bit unary where each lane's labels are an even count (aligned copies)
    const bool t16 = hpass && full && a.thetaq != nullptr && P % 2 == 0;
    const size_t sm = sizeof(float) * wpb * (size_t)ring_floats(P, RING, hpass, t16);
    if (sm > 227 * 1024) return fail(CNNCRF_EUNSUPPORTED, "crf: %zu bytes of ring per CTA", sm);
    auto kern = hpass ? (full ? k_crf_chain<P, DELTA, true, true, RING> : k_crf_chain<P, DELTA, true, false, RING>)
                      : (full ? k_crf_chain<P, DELTA, false, true, RING> : k_crf_chain<P, DELTA, false, false, RING>);
    if constexpr (P % 2 == 0)
        if (t16) kern = k_crf_chain<P, DELTA, true, true, RING, true>;
    // cooperative 16-byte copies where the vectors allow them (the workspace's phi and messages are 256-byte
    // aligned; a caller's cost volume may not be)
    {
        const bool aligned = (((uintptr_t)a.theta | (uintptr_t)a.thetaq | (uintptr_t)a.phi | (uintptr_t)a.lbuf) & 15) == 0;
        if (full && aligned) {
            if (!hpass) kern = k_crf_chain<P, DELTA, false, true, RING, false, true>;
            else if (t16) kern = k_crf_chain<P, DELTA, true, true, RING, P % 2 == 0, true>;
            else kern = k_crf_chain<P, DELTA, true, true, RING, false, true>;
        }
    }
    CNNCRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const long chains = (long)(hpass ? a.H : a.W) * a.np;
    {
        CNNCRF_PROF(hpass ? "crf_h" : "crf_v", st);
        kern<<<ceil_div(chains, wpb), 32 * wpb, sm, st>>>(a.theta, a.thetaq, a.qscale, a.qoffset23, a.phi, a.wgt,
                                                           a.lbuf, a.W, a.H, a.D, a.rp,
                                                           a.first, a.store_phi, a.labels, a.cmin, a.np,
                                                           a.wps);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

template <int P, int RING>
int launch_pass_delta(const CrfPassArgs &a, bool hpass, int delta, int wpb, cudaStream_t st)
{
    switch (delta) {
    case 1: return launch_pass<P, 1, RING>(a, hpass, wpb, st);
    case 2: return launch_pass<P, 2, RING>(a, hpass, wpb, st);
    case 3: return launch_pass<P, 3, RING>(a, hpass, wpb, st);
    case 4: return launch_pass<P, 4, RING>(a, hpass, wpb, st);
    default: return fail(CNNCRF_EUNSUPPORTED, "crf: delta %d outside 1..4", delta);
    }
}

// labels per lane P = ceil(D / 32) rounded up to 1, 2, 3, 4, 6 or 8
template <int RING>
int launch_pass_any(const CrfPassArgs &a, bool hpass, int delta, int wpb, cudaStream_t st)
{
    if (wpb < 1 || wpb > 4) return fail(CNNCRF_EINVAL, "crf: %d chains per CTA outside 1..4", wpb);
    const int P = (a.D + 31) / 32;
    if (P <= 1) return launch_pass_delta<1, RING>(a, hpass, delta, wpb, st);
    if (P <= 2) return launch_pass_delta<2, RING>(a, hpass, delta, wpb, st);
    if (P <= 3) return launch_pass_delta<3, RING>(a, hpass, delta, wpb, st);
    if (P <= 4) return launch_pass_delta<4, RING>(a, hpass, delta, wpb, st);
    if (P <= 6) return launch_pass_delta<6, RING>(a, hpass, delta, wpb, st);
    return launch_pass_delta<8, RING>(a, hpass, delta, wpb, st);
}

} // namespace

} // namespace k
} // namespace cnncrf

#endif
