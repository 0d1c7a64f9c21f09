// k_train.cu -- the kernels of the training step: weight layouts from the
// npz layout, the adjoints of tanh, the L2 normalisation, the correlation,
// the convolutions (weight gradient here, input gradient through conv_simt on
// the zero-padded output gradient) and the pairwise head, the structured
// hinge's subgradient and the SGD-with-momentum update.
//
// The reference ships no training code; its only gradient code is the
// correlation's backward (stereo/operators/stereocorrelation.cu:210-350),
// whose integer-disparity form the correlation adjoint here follows: dL/dfL
// and dL/dfR of C[y][x][k] = <fL(y, x), fR(y, x + s_k)>, zero where x + s_k
// leaves the row.  Everything is FP32 with fixed reduction orders (weight and
// bias gradients sum fixed pixel chunks, then the chunks in order), so a step
// is deterministic run to run.
#include <algorithm>
#include <cfloat>

#include <cuda_bf16.h>

#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

// activations are FP32 or BF16 (the BF16 training mode), read at a channel stride
__device__ __forceinline__ float ld(const float *p) { return *p; }
__device__ __forceinline__ float ld(const __nv_bfloat16 *p) { return __bfloat162float(*p); }

// ------------------------------------------------------------ weight layouts
// forward (conv_simt): wt[(ky*kw + kx)*Cin + ci][co] = w[co][ci][kh-1-ky][kw-1-kx], [K][128]
__global__ void k_w_fwd(const float *__restrict__ w, int Cout, int Cin, int kh, int kw, float *__restrict__ wt)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x, K = (long)kh * kw * Cin;
    if (i >= K * 128) return;
    const int k = (int)(i / 128), co = (int)(i % 128);
    const int ci = k % Cin, t = k / Cin, kx = t % kw, ky = t / kw;
    wt[i] = co < Cout ? w[(((long)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)] : 0.0f;
}

// input gradient as conv_simt on the output gradient padded by (kh-1, kw-1):
// wd[(ky*kw + kx)*Cout + co][ci] = w[co][ci][ky][kx], [kh*kw*Cout][128]
__global__ void k_w_dgrad(const float *__restrict__ w, int Cout, int Cin, int kh, int kw, float *__restrict__ wd)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x, K = (long)kh * kw * Cout;
    if (i >= K * 128) return;
    const int k = (int)(i / 128), ci = (int)(i % 128);
    const int co = k % Cout, t = k / Cout, kx = t % kw, ky = t / kw;
    wd[i] = ci < Cin ? w[(((long)co * Cin + ci) * kh + ky) * kw + kx] : 0.0f;
}

// tensor-core conv (conv_tc): w16[(co*kh*kw + ky*kw + kx)*cp + ci] = bf16(w[co][ci][kh-1-ky][kw-1-kx]),
// [np][kh*kw][cp], zero past Cout / Cin
__global__ void k_w16(const float *__restrict__ w, int Cout, int Cin, int kh, int kw, int np, int cp,
                      __nv_bfloat16 *__restrict__ w16)
{
    const long taps = (long)kh * kw, i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)np * taps * cp) return;
    const int ci = (int)(i % cp);
    const long r = i / cp;
    const int t = (int)(r % taps), co = (int)(r / taps), ky = t / kw, kx = t % kw;
    const float v = (co < Cout && ci < Cin) ? w[(((long)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)] : 0.0f;
    w16[i] = __float2bfloat16_rn(v);
}

// the input gradient's tensor-core layout: w16d[ci][ky][kx][co] = w[co][ci][ky][kx]
// (transposed, not flipped: the gradient is the valid convolution of the
// (kh-1, kw-1)-padded output gradient with the unflipped kernel), zero padded
// to [np][kh*kw][cp]
__global__ void k_w16_dgrad(const float *__restrict__ w, int Cout, int Cin, int kh, int kw, int np, int cp,
                            __nv_bfloat16 *__restrict__ w16d)
{
    const long taps = (long)kh * kw, i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)np * taps * cp) return;
    const int co = (int)(i % cp);
    const long r = i / cp;
    const int t = (int)(r % taps), ci = (int)(r / taps), ky = t / kw, kx = t % kw;
    const float v = (ci < Cin && co < Cout) ? w[(((long)co * Cin + ci) * kh + ky) * kw + kx] : 0.0f;
    w16d[i] = __float2bfloat16_rn(v);
}


// pw = |h|, h[o] = sum_c wh[o][c] y2[c] on BF16 y2 (channel stride cs): [img][2][npx]
__global__ void k_head2_bf16(const __nv_bfloat16 *__restrict__ y2, int npx, int P, int cs, const float *__restrict__ wh,
                             float *__restrict__ out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x, img = blockIdx.y;
    if (p >= npx) return;
    const __nv_bfloat16 *v = y2 + ((long)img * npx + p) * cs;
    float h0 = 0.0f, h1 = 0.0f;
    for (int c = 0; c < P; ++c) {
        const float x = ld(v + c);
        h0 = fmaf(wh[c], x, h0);
        h1 = fmaf(wh[P + c], x, h1);
    }
    out[(long)img * 2 * npx + p] = fabsf(h0);
    out[((long)img * 2 + 1) * npx + p] = fabsf(h1);
}

__global__ void k_pad128(const float *__restrict__ b, int n, float *__restrict__ out)
{
    const int i = threadIdx.x;
    if (i < 128) out[i] = i < n ? b[i] : 0.0f;
}

// ------------------------------------------------------------ elementwise
template <class T>
__global__ void k_tanh_bwd(float *__restrict__ dy, const T *__restrict__ y, long npx, int C, int ys)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npx * C) {
        const float v = ld(y + (i / C) * ys + i % C);
        dy[i] = dy[i] * (1.0f - v * v);
    }
}

// dz = dy * (1 - y^2) in place (dense FP32 [n][H][W][C], y BF16 at channel
// stride ys), and its BF16 copy with a zero border of p rows and q columns and
// channels zero padded to cp: [n][H + 2p][W + 2q][cp].  A thread per padded
// pixel and 8-channel group (one 16-byte store).
__global__ void k_tanh_bwd_pad(float *__restrict__ dy, const __nv_bfloat16 *__restrict__ y, int H, int W, int C,
                               int ys, int p, int q, int cp, long total, __nv_bfloat16 *__restrict__ out)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int groups = cp >> 3, g = (int)(i % groups);
    const long px = i / groups;
    const int Wp = W + 2 * q, Hp = H + 2 * p;
    const int xp = (int)(px % Wp);
    const long r = px / Wp;
    const int yp = (int)(r % Hp), img = (int)(r / Hp);
    const int x = xp - q, yy = yp - p;
    uint32_t u[4] = {0u, 0u, 0u, 0u};
    if (x >= 0 && x < W && yy >= 0 && yy < H) {
        const long pix = ((long)img * H + yy) * W + x;
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = g * 8 + j;
            v[j] = 0.0f;
            if (c < C) {
                const float a = __bfloat162float(y[pix * ys + c]);
                v[j] = dy[pix * C + c] * (1.0f - a * a);
                dy[pix * C + c] = v[j];
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
            u[j] = *(uint32_t *)&b2;
        }
    }
    *(uint4 *)(out + px * cp + g * 8) = make_uint4(u[0], u[1], u[2], u[3]);
}

// zero the border pixels of [n][H + 2p][W + 2q][cp] BF16: a thread per (border pixel, 8-channel group)
__global__ void k_zero_border(__nv_bfloat16 *__restrict__ buf, int H, int W, int cp, int p, int q, long per_img,
                              long total)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const int groups = cp >> 3, g = (int)(i % groups);
    const long b = i / groups;
    const int img = (int)(b / per_img);
    long r = b - img * per_img; // border pixel index within the image
    const int Wp = W + 2 * q, Hp = H + 2 * p;
    int yy, xx;
    if (r < (long)p * Wp) { // top rows
        yy = (int)(r / Wp), xx = (int)(r % Wp);
    } else if ((r -= (long)p * Wp) < (long)p * Wp) { // bottom rows
        yy = H + p + (int)(r / Wp), xx = (int)(r % Wp);
    } else { // left and right columns of the middle rows
        r -= (long)p * Wp;
        const int side = (int)(r / ((long)H * q));
        r -= (long)side * H * q;
        yy = p + (int)(r / q), xx = (int)(r % q) + (side ? W + q : 0);
    }
    *(uint4 *)(buf + (((long)img * Hp + yy) * Wp + xx) * cp + g * 8) = make_uint4(0u, 0u, 0u, 0u);
}

// out [n][H + 2p][W + 2q][C] = in [n][H][W][C] with a zero border
__global__ void k_pad_zero(const float *__restrict__ in, int H, int W, int C, int p, int q, float *__restrict__ out)
{
    const int Hp = H + 2 * p, Wp = W + 2 * q;
    const long per = (long)Hp * Wp * C;
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const int img = blockIdx.y;
    if (i >= per) return;
    const int c = (int)(i % C);
    const long px = i / C;
    const int x = (int)(px % Wp) - q, y = (int)(px / Wp) - p;
    out[(long)img * per + i] =
        (x >= 0 && x < W && y >= 0 && y < H) ? in[(((long)img * H + y) * W + x) * C + c] : 0.0f;
}

// f = y / |y| per pixel; dy = (df - y <y, df> / |y|^2) / |y|, zero where |y| = 0.  A warp per pixel.
template <class T>
__global__ void k_l2norm_bwd(const T *__restrict__ y, int ys, const float *__restrict__ df, long npx, int C,
                             float *__restrict__ dy)
{
    const long px = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (px >= npx) return;
    const T *yp = y + px * ys;
    const float *gp = df + px * C;
    float ss = 0.0f, dot = 0.0f;
    for (int c = lane; c < C; c += 32) {
        ss = fmaf(ld(yp + c), ld(yp + c), ss);
        dot = fmaf(ld(yp + c), gp[c], dot);
    }
    for (int o = 16; o; o >>= 1) {
        ss += __shfl_xor_sync(0xffffffffu, ss, o);
        dot += __shfl_xor_sync(0xffffffffu, dot, o);
    }
    const float n = sqrtf(ss);
    for (int c = lane; c < C; c += 32)
        dy[px * C + c] = n > 0.0f ? (gp[c] - ld(yp + c) * (dot / ss)) / n : 0.0f;
}

// The last feature layer's whole output gradient in one pass (BF16 mode):
//   dy = (df - y <y, df> / |y|^2) / |y|   (the L2 normalisation's adjoint, zero where |y| = 0)
//   dz = dy (1 - y^2)                     (tanh')
// written as BF16 into [n][H + 2p][W + 2q][128] inside its border, and the
// CTA's per-channel sums of dz into part[blockIdx.x][C] (warp sums added in
// warp order).  A warp per pixel, lane l channels 4l .. 4l + 3, four pixels
// per warp in flight; C <= 128, C and ys multiples of 4.
__global__ void __launch_bounds__(256) k_l2norm_tanh_bwd_pad(const __nv_bfloat16 *__restrict__ y, int ys,
                                                             const float *__restrict__ df, int H, int W, int C,
                                                             long npx, int p, int q, __nv_bfloat16 *__restrict__ out,
                                                             float *__restrict__ part)
{
    __shared__ float ws[8][128];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, c0 = 4 * lane;
    const long nw = (long)gridDim.x * 8;
    float bs[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (long px0 = (long)blockIdx.x * 8 + w; px0 < npx; px0 += 4 * nw) {
        float yq[4][4], gq[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) { // the loads of four pixels first
            const long px = px0 + u * nw;
            uint2 yr = make_uint2(0u, 0u);
            float4 gr = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (px < npx && c0 < C) {
                yr = *(const uint2 *)(y + px * ys + c0);
                gr = *(const float4 *)(df + px * C + c0);
            }
            yq[u][0] = __uint_as_float(yr.x << 16), yq[u][1] = __uint_as_float(yr.x & 0xffff0000u);
            yq[u][2] = __uint_as_float(yr.y << 16), yq[u][3] = __uint_as_float(yr.y & 0xffff0000u);
            gq[u][0] = gr.x, gq[u][1] = gr.y, gq[u][2] = gr.z, gq[u][3] = gr.w;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long px = px0 + u * nw;
            if (px >= npx) break; // warp-uniform
            const float *yv = yq[u], *g = gq[u];
            float ss = 0.0f, dot = 0.0f;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                ss = fmaf(yv[j], yv[j], ss);
                dot = fmaf(yv[j], g[j], dot);
            }
            for (int o = 16; o; o >>= 1) {
                ss += __shfl_xor_sync(0xffffffffu, ss, o);
                dot += __shfl_xor_sync(0xffffffffu, dot, o);
            }
            const float n = sqrtf(ss), s = dot / ss, rn = 1.0f / n;
            float dz[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float d = n > 0.0f ? (g[j] - yv[j] * s) * rn : 0.0f;
                dz[j] = d * (1.0f - yv[j] * yv[j]);
                bs[j] += dz[j];
            }
            // 32-bit index arithmetic (npx < 2^31): 64-bit division is a long software sequence
            const unsigned pu = (unsigned)px, hw = (unsigned)H * W;
            const unsigned img = pu / hw, r = pu - img * hw, yy = r / W, x = r - yy * W;
            const long o = (((long)img * (H + 2 * p) + yy + p) * (W + 2 * q) + x + q) * 128 + c0;
            __nv_bfloat162 a = __floats2bfloat162_rn(dz[0], dz[1]), b = __floats2bfloat162_rn(dz[2], dz[3]);
            *(uint2 *)(out + o) = make_uint2(*(uint32_t *)&a, *(uint32_t *)&b);
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) ws[w][c0 + j] = bs[j];
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += 256) {
        float s = ws[0][c];
        for (int k = 1; k < 8; ++k) s += ws[k][c];
        part[(long)blockIdx.x * C + c] = s;
    }
}

// ------------------------------------------------------------ correlation adjoint
// Left: dfl[x][c] = -sum_k gvol[x][k] fr[x + s_k][c].  A CTA per (32-pixel
// tile, row, pair); thread c; the right features of the tile's band in shared memory.
template <class T>
__global__ void k_corr_bwd_left(const T *__restrict__ fr, int fs, const float *__restrict__ gvol,
                                const float *__restrict__ list, int H, int W, int C, int D, int omin, int span,
                                float *__restrict__ dfl)
{
    extern __shared__ float win[]; // [span][C], column j = pixel x0 + omin + j
    int *s = (int *)(win + (size_t)span * C);
    const int x0 = blockIdx.x * 32, y = blockIdx.y, pair = blockIdx.z;
    const long row = ((long)pair * H + y) * W;
    for (int i = threadIdx.x; i < D; i += blockDim.x) s[i] = (int)list[i];
    for (int i = threadIdx.x; i < span * C; i += blockDim.x) {
        const int xs = x0 + omin + i / C, c = i % C;
        win[i] = (xs >= 0 && xs < W) ? ld(fr + (row + xs) * fs + c) : 0.0f;
    }
    __syncthreads();
    const int c = threadIdx.x;
    if (c >= C) return;
    for (int i = 0; i < 32 && x0 + i < W; ++i) {
        const int x = x0 + i;
        const float *g = gvol + (row + x) * D;
        float acc = 0.0f;
        for (int k = 0; k < D; ++k) {
            const int xs = x + s[k];
            if (xs >= 0 && xs < W) acc = fmaf(g[k], win[(size_t)(xs - x0 - omin) * C + c], acc);
        }
        dfl[(row + x) * C + c] = -acc;
    }
}

// Right: dfr[x'][c] = -sum_k gvol[x' - s_k][k] fl[x' - s_k][c] over x' - s_k in
// [0, W); the left features x' - omax .. x' + 31 - omin in shared memory.
template <class T>
__global__ void k_corr_bwd_right(const T *__restrict__ fl, int fs, const float *__restrict__ gvol,
                                 const float *__restrict__ list, int H, int W, int C, int D, int omax, int span,
                                 float *__restrict__ dfr)
{
    extern __shared__ float win[]; // [span][C], column j = pixel x0 - omax + j
    int *s = (int *)(win + (size_t)span * C);
    const int x0 = blockIdx.x * 32, y = blockIdx.y, pair = blockIdx.z;
    const long row = ((long)pair * H + y) * W;
    for (int i = threadIdx.x; i < D; i += blockDim.x) s[i] = (int)list[i];
    for (int i = threadIdx.x; i < span * C; i += blockDim.x) {
        const int x = x0 - omax + i / C, c = i % C;
        win[i] = (x >= 0 && x < W) ? ld(fl + (row + x) * fs + c) : 0.0f;
    }
    __syncthreads();
    const int c = threadIdx.x;
    if (c >= C) return;
    for (int i = 0; i < 32 && x0 + i < W; ++i) {
        const int xr = x0 + i;
        float acc = 0.0f;
        for (int k = 0; k < D; ++k) {
            const int x = xr - s[k];
            if (x >= 0 && x < W) acc = fmaf(gvol[(row + x) * D + k], win[(size_t)(x - x0 + omax) * C + c], acc);
        }
        dfr[(row + xr) * C + c] = -acc;
    }
}

// Both sides as one banded product, blocked in registers:
//   dF[u][c] = -sum_k a(u, k) F[u + o_k][c]
//   left  (right = 0): o_k =  s_k, a(u, k) = gvol[u][k],         F = fr
//   right (right = 1): o_k = -s_k, a(u, k) = gvol[u - s_k][k],   F = fl
// A CTA per (64-pixel tile, row, pair), 256 threads.  Shared memory holds the
// band matrix As[v][u] = a(u, k) at the partner pixel v = u + o_k (zero where
// no offset of the list lands; the offsets are distinct) for v in the window
// x0 + omn .. x0 + 63 + omn + span - 1, and the partner features Fs[v][c]
// (zero outside the row and past C).  Warp w owns pixels x0 + 8w .. + 7,
// lane l channels 4l .. 4l + 3: per partner pixel two broadcast loads of As,
// one load of Fs and 32 FMAs in FP32.
constexpr int CB_TX = 64, CB_AS = CB_TX + 4;

__device__ __forceinline__ void ld4(const float *p, float *f)
{
    const float4 v = *(const float4 *)p;
    f[0] = v.x, f[1] = v.y, f[2] = v.z, f[3] = v.w;
}
__device__ __forceinline__ void ld4(const __nv_bfloat16 *p, float *f)
{
    const uint2 v = *(const uint2 *)p;
    f[0] = __uint_as_float(v.x << 16), f[1] = __uint_as_float(v.x & 0xffff0000u);
    f[2] = __uint_as_float(v.y << 16), f[3] = __uint_as_float(v.y & 0xffff0000u);
}

size_t corr_bwd_blk_smem(int span, int Cs, size_t es, int D)
{
    const size_t nv = CB_TX - 1 + span;
    return nv * CB_AS * 4 + ((nv * Cs * es + 15) & ~(size_t)15) + 4 * (size_t)D;
}

template <class T>
__global__ void __launch_bounds__(256) k_corr_bwd_blk(const T *__restrict__ F, int fs, const float *__restrict__ gvol,
                                                      const float *__restrict__ list, int H, int W, int C, int Cs,
                                                      int D, int right, int omn, int span, float *__restrict__ out)
{
    extern __shared__ float4 smem4[];
    const int NV = CB_TX - 1 + span;
    float *As = (float *)smem4;
    T *Fs = (T *)(As + (size_t)NV * CB_AS);
    int *offs = (int *)((char *)Fs + (((size_t)NV * Cs * sizeof(T) + 15) & ~(size_t)15));
    const int tid = threadIdx.x, x0 = blockIdx.x * CB_TX, y = blockIdx.y, pair = blockIdx.z;
    const long row = ((long)pair * H + y) * W;
    const int vbase = x0 + omn;
    for (int k = tid; k < D; k += 256) offs[k] = right ? -(int)list[k] : (int)list[k];
    for (int i = tid; i < NV * CB_AS; i += 256) As[i] = 0.0f;
    for (int i = tid; i < NV * Cs; i += 256) {
        const int vr = i / Cs, c = i % Cs, x = vbase + vr;
        Fs[i] = (x >= 0 && x < W && c < C) ? F[(row + x) * fs + c] : T(0.0f);
    }
    __syncthreads();
    if (!right) {
        for (int i = tid; i < CB_TX * D; i += 256) {
            const int r = i / D, k = i % D, u = x0 + r;
            if (u < W) As[(r + offs[k] - omn) * CB_AS + r] = gvol[(row + u) * D + k];
        }
    } else {
        for (int i = tid; i < NV * D; i += 256) {
            const int r = i / D, k = i % D, x = vbase + r, ur = x - offs[k] - x0;
            if (x >= 0 && x < W && ur >= 0 && ur < CB_TX && x0 + ur < W) As[r * CB_AS + ur] = gvol[(row + x) * D + k];
        }
    }
    __syncthreads();
    const int u0 = (tid >> 5) * 8, c0 = (tid & 31) * 4;
    if (c0 >= C) return;
    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    const int v1 = u0 + 7 + span; // partner rows of pixels u0 .. u0 + 7
#pragma unroll 2
    for (int vr = u0; vr < v1; ++vr) {
        float a[8], f[4];
        ld4(As + vr * CB_AS + u0, a);
        ld4(As + vr * CB_AS + u0 + 4, a + 4);
        ld4(Fs + (size_t)vr * Cs + c0, f);
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], f[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int u = x0 + u0 + i;
        if (u < W)
#pragma unroll
            for (int j = 0; j < 4; ++j)
                if (c0 + j < C) out[(row + u) * C + c0 + j] = -acc[i][j];
    }
}

// ------------------------------------------------------------ weight gradient
// part[split][co][k] = sum over the split's pixels p of dz[p][co] * A[p][k],
// A[p][(ky*kw + kx)*Cin + ci] = in(img, oy + ky, ox + kx, ci).  A CTA per
// (64-wide k tile, split); 256 threads, 8 co x 4 k each; 32 pixels staged per step.
template <class T> struct WgradArgs {
    const float *dz;
    int Cout;
    const T *in;
    long in_pix, in_row, in_img;
    int Cin, kh, kw, Ho, Wo;
    long P, chunk;
    float *part;
};

constexpr int WG_PX = 32, WG_KT = 64;

template <class T> __global__ void __launch_bounds__(256) k_wgrad(const WgradArgs<T> a)
{
    __shared__ float As[WG_PX][128];
    __shared__ float Bs[WG_PX][WG_KT];
    const int K = a.kh * a.kw * a.Cin;
    const int kt0 = blockIdx.x * WG_KT, split = blockIdx.y;
    const long p0 = (long)split * a.chunk, p1 = min(a.P, p0 + a.chunk);
    const int t = threadIdx.x, cb = (t & 15) * 8, kb = (t >> 4) * 4;
    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0f;
    for (long pb = p0; pb < p1; pb += WG_PX) {
        for (int i = t; i < WG_PX * 128; i += 256) {
            const int pp = i / 128, co = i % 128;
            const long p = pb + pp;
            As[pp][co] = (p < p1 && co < a.Cout) ? a.dz[p * a.Cout + co] : 0.0f;
        }
        for (int i = t; i < WG_PX * WG_KT; i += 256) {
            const int pp = i / WG_KT, kk = kt0 + i % WG_KT;
            const long p = pb + pp;
            float v = 0.0f;
            if (p < p1 && kk < K) {
                const int ci = kk % a.Cin, tt = kk / a.Cin, kx = tt % a.kw, ky = tt / a.kw;
                const long img = p / ((long)a.Ho * a.Wo), r = p - img * a.Ho * a.Wo;
                const int oy = (int)(r / a.Wo), ox = (int)(r % a.Wo);
                v = ld(a.in + img * a.in_img + (long)(oy + ky) * a.in_row + (long)(ox + kx) * a.in_pix + ci);
            }
            Bs[pp][i % WG_KT] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int pp = 0; pp < WG_PX; ++pp) {
            float av[8], bv[4];
#pragma unroll
            for (int i = 0; i < 8; ++i) av[i] = As[pp][cb + i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[pp][kb + j];
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int co = cb + i, kk = kt0 + kb + j;
            if (co < a.Cout && kk < K) a.part[((long)split * a.Cout + co) * K + kk] = acc[i][j];
        }
}

// dw[co][ci][kh-1-ky][kw-1-kx] += sum_split part[split][co][k], splits in order
// dw (npz layout) += the sum over splits of part[split][co][k]: 32 outputs
// per CTA (one per lane), warp w sums splits w, w + 8, ..., then lane sums of
// the 8 warps in a fixed order (deterministic)
__global__ void __launch_bounds__(256) k_wgrad_reduce(const float *__restrict__ part, int nsplit, int Cout, int Cin,
                                                      int kh, int kw, float *__restrict__ dw)
{
    __shared__ float s[8][33];
    const int K = kh * kw * Cin, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long n = (long)Cout * K, i = (long)blockIdx.x * 32 + lane;
    float acc = 0.0f;
    if (i < n)
        for (int sp = w; sp < nsplit; sp += 8) acc += part[(long)sp * n + i];
    s[w][lane] = acc;
    __syncthreads();
    if (w != 0 || i >= n) return;
    float t = s[0][lane];
#pragma unroll
    for (int j = 1; j < 8; ++j) t += s[j][lane];
    const int co = (int)(i / K), k = (int)(i % K);
    const int ci = k % Cin, tt = k / Cin, kx = tt % kw, ky = tt / kw;
    dw[(((long)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)] += t;
}

// db[co] += sum_p dz[p][co]: per split a partial, then the splits in order
// A CTA of 128 x 4 threads per split: thread (co, r) sums the split's pixels
// r, r + 4, ...; the 4 sums are added in order.
__global__ void __launch_bounds__(512) k_bias_part(const float *__restrict__ dz, int Cout, long P, long chunk,
                                                   float *__restrict__ part)
{
    __shared__ float s4[4][128];
    const int co = threadIdx.x, r = threadIdx.y, split = blockIdx.x;
    const long p0 = (long)split * chunk, p1 = min(P, p0 + chunk);
    float s = 0.0f;
    if (co < Cout)
#pragma unroll 4
        for (long p = p0 + r; p < p1; p += 4) s += dz[p * Cout + co];
    s4[r][co] = s;
    __syncthreads();
    if (r == 0 && co < Cout) part[(long)split * Cout + co] = ((s4[0][co] + s4[1][co]) + s4[2][co]) + s4[3][co];
}

// db[co] += the sum over splits: warp w sums splits w, w + 8, ... of 32
// channels, then the 8 warp sums in order
__global__ void __launch_bounds__(256) k_bias_reduce(const float *__restrict__ part, int nsplit, int Cout,
                                                     float *__restrict__ db)
{
    __shared__ float s8[8][33];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, co = blockIdx.x * 32 + lane;
    float s = 0.0f;
    if (co < Cout)
        for (int sp = w; sp < nsplit; sp += 8) s += part[(long)sp * Cout + co];
    s8[w][lane] = s;
    __syncthreads();
    if (w != 0 || co >= Cout) return;
    float t = s8[0][lane];
#pragma unroll
    for (int j = 1; j < 8; ++j) t += s8[j][lane];
    db[co] += t;
}

// BF16 copy of an FP32 [npx][C] image with channels padded to 64: the
// tensor-core weight gradient's operand for the thin first layers
__global__ void k_to_bf16_c64(const float *__restrict__ in, long npx, int C, __nv_bfloat16 *__restrict__ out)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x; // one 8-channel group
    if (i >= npx * 8) return;
    const long px = i >> 3;
    const int g = (int)(i & 7);
    uint32_t u[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int c0 = g * 8 + 2 * j, c1 = c0 + 1;
        __nv_bfloat162 b2 = __floats2bfloat162_rn(c0 < C ? in[px * C + c0] : 0.0f, c1 < C ? in[px * C + c1] : 0.0f);
        u[j] = *(uint32_t *)&b2;
    }
    *(uint4 *)(out + px * 64 + g * 8) = make_uint4(u[0], u[1], u[2], u[3]);
}

// The 1x1 head's weight gradient: part[split][o][c] = sum over the split's
// pixels of gh[p][o] y[p][c], o < 2; thread (c, o, r) takes pixels r, r + 2, ...
template <class T>
__global__ void __launch_bounds__(512) k_wgrad_head(const float *__restrict__ gh, const T *__restrict__ y, int ys,
                                                    long P, long chunk, int C, float *__restrict__ part)
{
    __shared__ float s2[2][2][128];
    const int c = threadIdx.x, o = threadIdx.y, r = threadIdx.z, split = blockIdx.x;
    const long p0 = (long)split * chunk, p1 = min(P, p0 + chunk);
    float s = 0.0f;
    if (c < C)
#pragma unroll 4
        for (long p = p0 + r; p < p1; p += 2) s = fmaf(gh[p * 2 + o], ld(y + p * ys + c), s);
    s2[r][o][c] = s;
    __syncthreads();
    if (r == 0 && c < C) part[((long)split * 2 + o) * C + c] = s2[0][o][c] + s2[1][o][c];
}

// ------------------------------------------------------------ pairwise head adjoint
// pw = |h|, h[o] = sum_c wh[o][c] y2[c]: gh[o] = gpw[o] sign(h[o]); dy2[c] = sum_o wh[o][c] gh[o]
template <class T>
__global__ void k_head_bwd(const T *__restrict__ y2, int ys, const float *__restrict__ wh, const float *__restrict__ gpw,
                           int npx, int P, float *__restrict__ gh, float *__restrict__ dy2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x, img = blockIdx.y;
    if (p >= npx) return;
    const long q = (long)img * npx + p;
    const T *v = y2 + q * ys;
    float h0 = 0.0f, h1 = 0.0f;
    for (int c = 0; c < P; ++c) {
        h0 = fmaf(wh[c], ld(v + c), h0);
        h1 = fmaf(wh[P + c], ld(v + c), h1);
    }
    const float a0 = gpw[(long)img * 2 * npx + p], a1 = gpw[((long)img * 2 + 1) * npx + p];
    const float g0 = h0 > 0.0f ? a0 : (h0 < 0.0f ? -a0 : 0.0f);
    const float g1 = h1 > 0.0f ? a1 : (h1 < 0.0f ? -a1 : 0.0f);
    gh[q * 2] = g0;
    gh[q * 2 + 1] = g1;
    for (int c = 0; c < P; ++c) dy2[q * P + c] = fmaf(wh[c], g0, wh[P + c] * g1);
}

// The head's adjoint and the second pairwise layer's tanh' in one pass (BF16
// mode, P <= 64): gh = gpw sign(h), dz = (W^T gh)(1 - y2^2), dz written as
// BF16 into [n][H + 2p][W + 2q][64] inside its border, gh as FP32 [px][2], and
// the CTA's per-channel sums of dz into part[blockIdx.x][P].  A warp per pixel,
// lane l channels 2l, 2l + 1; four pixels per warp in flight.
__global__ void __launch_bounds__(256) k_head_tanh_bwd_pad(const __nv_bfloat16 *__restrict__ y2, int ys,
                                                           const float *__restrict__ wh, const float *__restrict__ gpw,
                                                           int H, int W, int P, long npx, int p, int q,
                                                           float *__restrict__ gh, __nv_bfloat16 *__restrict__ out,
                                                           float *__restrict__ part)
{
    __shared__ float ws[8][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, c0 = 2 * lane;
    const bool on = c0 < P;
    const float w00 = on ? wh[c0] : 0.0f, w01 = on && c0 + 1 < P ? wh[c0 + 1] : 0.0f;
    const float w10 = on ? wh[P + c0] : 0.0f, w11 = on && c0 + 1 < P ? wh[P + c0 + 1] : 0.0f;
    const long nw = (long)gridDim.x * 8, hw = (long)H * W;
    float b0 = 0.0f, b1 = 0.0f;
    for (long px0 = (long)blockIdx.x * 8 + w; px0 < npx; px0 += 4 * nw) {
        uint32_t yr[4];
        float a0[4], a1[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) { // the loads of four pixels first
            const long px = px0 + u * nw;
            yr[u] = 0u, a0[u] = 0.0f, a1[u] = 0.0f;
            if (px < npx) {
                if (on) yr[u] = *(const uint32_t *)(y2 + px * ys + c0);
                const unsigned img = (unsigned)px / (unsigned)hw, r = (unsigned)px - img * (unsigned)hw;
                a0[u] = gpw[(long)(img * 2) * hw + r], a1[u] = gpw[(long)(img * 2 + 1) * hw + r];
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long px = px0 + u * nw;
            if (px >= npx) break; // warp-uniform
            const float ya = __uint_as_float(yr[u] << 16), yb = __uint_as_float(yr[u] & 0xffff0000u);
            float h0 = fmaf(w00, ya, w01 * yb), h1 = fmaf(w10, ya, w11 * yb);
            for (int o = 16; o; o >>= 1) {
                h0 += __shfl_xor_sync(0xffffffffu, h0, o);
                h1 += __shfl_xor_sync(0xffffffffu, h1, o);
            }
            const float g0 = h0 > 0.0f ? a0[u] : (h0 < 0.0f ? -a0[u] : 0.0f);
            const float g1 = h1 > 0.0f ? a1[u] : (h1 < 0.0f ? -a1[u] : 0.0f);
            if (lane == 0) *(float2 *)(gh + px * 2) = make_float2(g0, g1);
            const float da = fmaf(w00, g0, w10 * g1) * (1.0f - ya * ya);
            const float db = fmaf(w01, g0, w11 * g1) * (1.0f - yb * yb);
            b0 += da, b1 += db;
            const unsigned img = (unsigned)px / (unsigned)hw, r = (unsigned)px - img * (unsigned)hw;
            const unsigned yy = r / W, x = r - yy * W;
            __nv_bfloat162 d2 = __floats2bfloat162_rn(da, db);
            if (c0 < 64)
                *(uint32_t *)(out + (((long)img * (H + 2 * p) + yy + p) * (W + 2 * q) + x + q) * 64 + c0) =
                    *(uint32_t *)&d2;
        }
    }
    ws[w][c0] = b0, ws[w][c0 + 1] = b1;
    __syncthreads();
    for (int c = threadIdx.x; c < P; c += 256) {
        float s = ws[0][c];
        for (int k = 1; k < 8; ++k) s += ws[k][c];
        part[(long)blockIdx.x * P + c] = s;
    }
}

// ------------------------------------------------------------ structured hinge
// aug = vol, + 1 at the ground-truth label (invalid labels: counted in err, left out)
// a warp per pixel (grid-stride), lane l the labels 4l + 128 j: no index division
__global__ void k_augment(const float *__restrict__ vol, const int32_t *__restrict__ gt, long npx, int D,
                          float *__restrict__ aug, int *__restrict__ err)
{
    const int lane = threadIdx.x & 31;
    const long nw = ((long)gridDim.x * blockDim.x) >> 5;
    for (long px = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; px < npx; px += nw) {
        const int g = gt[px];
        if (lane == 0 && (g < 0 || g >= D)) atomicAdd(err, 1);
        const float *v = vol + px * D;
        float *a = aug + px * D;
        if ((D & 3) == 0) {
            for (int k = 4 * lane; k < D; k += 128) {
                float4 x = *(const float4 *)(v + k);
                x.x = g == k ? x.x + 1.0f : x.x;
                x.y = g == k + 1 ? x.y + 1.0f : x.y;
                x.z = g == k + 2 ? x.z + 1.0f : x.z;
                x.w = g == k + 3 ? x.w + 1.0f : x.w;
                *(float4 *)(a + k) = x;
            }
        } else {
            for (int k = lane; k < D; k += 32) a[k] = k == g ? v[k] + 1.0f : v[k];
        }
    }
}

__device__ __forceinline__ float rho_of(const float *rho, int delta, float L2, int t)
{
    t = t < 0 ? -t : t;
    return t == 0 ? 0.0f : (t <= delta ? rho[t] : L2);
}

struct HingeArgs {
    const float *vol, *w; // unary volume, lambda * pw ([n][2][H][W])
    const int32_t *gt, *yh;
    int W, H, D;
    float lam, L2;
    int delta;
    float rho[9];
    float gscale;      // scale of the subgradient (1, or 1 / pixels of the batch for the mean loss)
    float *gvol, *gpw; // gvol zeroed by the caller
    double *contrib;   // per pixel: its unary, margin and right / down edge terms of E(gt) - E(yh) + margin
};

__global__ void k_hinge(const HingeArgs a)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y, img = blockIdx.z;
    if (x >= a.W) return;
    const long N = (long)a.W * a.H, i = (long)y * a.W + x, q = (long)img * N + i;
    const int g = a.gt[q], h = a.yh[q];
    float gx = 0.0f, gy = 0.0f;
    double c = 0.0;
    if (g >= 0 && g < a.D && h >= 0 && h < a.D) { // invalid labels are reported by k_augment
        float *gv = a.gvol + q * a.D;
        gv[g] += a.gscale;
        gv[h] -= a.gscale;
        c = (double)a.vol[q * a.D + g] - (double)a.vol[q * a.D + h] + (g != h ? 1.0 : 0.0);
        const float *wx = a.w + (long)img * 2 * N, *wy = wx + N;
        if (x + 1 < a.W) {
            const int g2 = a.gt[q + 1], h2 = a.yh[q + 1];
            if (g2 >= 0 && g2 < a.D && h2 >= 0 && h2 < a.D) {
                const float rg = rho_of(a.rho, a.delta, a.L2, g - g2), rh = rho_of(a.rho, a.delta, a.L2, h - h2);
                gx = a.lam * (rg - rh) * a.gscale;
                c += (double)wx[i] * (double)rg - (double)wx[i] * (double)rh;
            }
        }
        if (y + 1 < a.H) {
            const int g2 = a.gt[q + a.W], h2 = a.yh[q + a.W];
            if (g2 >= 0 && g2 < a.D && h2 >= 0 && h2 < a.D) {
                const float rg = rho_of(a.rho, a.delta, a.L2, g - g2), rh = rho_of(a.rho, a.delta, a.L2, h - h2);
                gy = a.lam * (rg - rh) * a.gscale;
                c += (double)wy[i] * (double)rg - (double)wy[i] * (double)rh;
            }
        }
    }
    a.gpw[(long)img * 2 * N + i] = gx;
    a.gpw[((long)img * 2 + 1) * N + i] = gy;
    a.contrib[q] = c;
}

// rows[r] = sum of row r's W contributions, left to right
__global__ void k_row_sums_d(const double *__restrict__ c, long rows, int W, double *__restrict__ out)
{
    const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double s = 0.0;
    for (int x = 0; x < W; ++x) s += c[r * W + x];
    out[r] = s;
}

// ------------------------------------------------------------ SGD with momentum
// v = mu v + g; theta -= lr v (the torch.optim.SGD convention, no dampening)
__global__ void k_sgd(float *__restrict__ theta, const float *__restrict__ g, float *__restrict__ v, long n,
                      float lr, float mu)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float nv = fmaf(mu, v[i], g[i]);
    v[i] = nv;
    theta[i] = fmaf(-lr, nv, theta[i]);
}

} // namespace

int train_weight_layouts(const float *w, const float *b, int Cout, int Cin, int kh, int kw, float *wt, float *wd,
                         float *b128, cudaStream_t st)
{
    const long K = (long)kh * kw * Cin, Kd = (long)kh * kw * Cout;
    if (wt) k_w_fwd<<<ceil_div(K * 128, 256), 256, 0, st>>>(w, Cout, Cin, kh, kw, wt);
    if (wd) k_w_dgrad<<<ceil_div(Kd * 128, 256), 256, 0, st>>>(w, Cout, Cin, kh, kw, wd);
    if (b && b128) k_pad128<<<1, 128, 0, st>>>(b, Cout, b128);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_w16(const float *w, int Cout, int Cin, int kh, int kw, int np, int cp, void *w16, cudaStream_t st)
{
    const long n = (long)np * kh * kw * cp;
    k_w16<<<ceil_div(n, 256), 256, 0, st>>>(w, Cout, Cin, kh, kw, np, cp, (__nv_bfloat16 *)w16);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_w16_dgrad(const float *w, int Cout, int Cin, int kh, int kw, int np, int cp, void *w16d, cudaStream_t st)
{
    const long n = (long)np * kh * kw * cp;
    k_w16_dgrad<<<ceil_div(n, 256), 256, 0, st>>>(w, Cout, Cin, kh, kw, np, cp, (__nv_bfloat16 *)w16d);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_tanh_bwd_pad(float *dy, const void *y, int nimg, int H, int W, int C, int ys, int p, int q, int cp,
                       void *out, cudaStream_t st)
{
    if (cp % 8 || cp < C || ((uintptr_t)out & 15)) return fail(CNNCRF_EINVAL, "tanh_bwd_pad: channel padding");
    const long total = (long)nimg * (H + 2 * p) * (W + 2 * q) * (cp / 8);
    {
        CNNCRF_PROF("tanh_bwd", st);
        k_tanh_bwd_pad<<<ceil_div(total, 256), 256, 0, st>>>(dy, (const __nv_bfloat16 *)y, H, W, C, ys, p, q, cp,
                                                             total, (__nv_bfloat16 *)out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_zero_border(void *buf, int nimg, int H, int W, int cp, int p, int q, cudaStream_t st)
{
    if (cp % 8 || ((uintptr_t)buf & 15)) return fail(CNNCRF_EINVAL, "zero_border: channel padding");
    const long per_img = 2L * p * (W + 2 * q) + 2L * H * q;
    const long total = (long)nimg * per_img * (cp / 8);
    if (total == 0) return CNNCRF_OK;
    k_zero_border<<<ceil_div(total, 256), 256, 0, st>>>((__nv_bfloat16 *)buf, H, W, cp, p, q, per_img, total);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_head2_bf16(const void *y2, int nimg, int npx, int P, int cs, const float *wh, float *out, cudaStream_t st)
{
    {
        CNNCRF_PROF("head2", st);
        k_head2_bf16<<<dim3(ceil_div(npx, 128), nimg), 128, 0, st>>>((const __nv_bfloat16 *)y2, npx, P, cs, wh, out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_tanh_bwd(float *dy, const void *y, bool bf16, long npx, int C, int ys, cudaStream_t st)
{
    {
        CNNCRF_PROF("tanh_bwd", st);
        if (bf16)
            k_tanh_bwd<<<ceil_div(npx * C, 256), 256, 0, st>>>(dy, (const __nv_bfloat16 *)y, npx, C, ys);
        else
            k_tanh_bwd<<<ceil_div(npx * C, 256), 256, 0, st>>>(dy, (const float *)y, npx, C, ys);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_pad_zero(const float *in, int nimg, int H, int W, int C, int p, int q, float *out, cudaStream_t st)
{
    const long per = (long)(H + 2 * p) * (W + 2 * q) * C;
    k_pad_zero<<<dim3(ceil_div(per, 256), nimg), 256, 0, st>>>(in, H, W, C, p, q, out);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_l2norm_bwd(const void *y, bool bf16, int ys, const float *df, long npx, int C, float *dy, cudaStream_t st)
{
    {
        CNNCRF_PROF("l2norm_bwd", st);
        if (bf16)
            k_l2norm_bwd<<<ceil_div(npx * 32, 256), 256, 0, st>>>((const __nv_bfloat16 *)y, ys, df, npx, C, dy);
        else
            k_l2norm_bwd<<<ceil_div(npx * 32, 256), 256, 0, st>>>((const float *)y, ys, df, npx, C, dy);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_l2norm_tanh_bwd_pad(const void *y, int ys, const float *df, int nimg, int H, int W, int C, int p, int q,
                              void *out, float *part, int *nsplit, cudaStream_t st)
{
    if (C > 128 || C % 4 || ys % 4 || ((uintptr_t)out & 15) || ((uintptr_t)y & 7) || ((uintptr_t)df & 15) ||
        (long)nimg * H * W >= (1L << 31))
        return fail(CNNCRF_EINVAL, "l2norm_tanh_bwd_pad: %d channels / layout", C);
    int dev = 0, sms = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long npx = (long)nimg * H * W;
    int per_sm = 1; // one full wave of resident CTAs (at most 4 per SM: the sums' rows)
    CNNCRF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_l2norm_tanh_bwd_pad, 256, 0));
    const int grid = (int)std::max(1L, std::min((long)std::min(4, std::max(1, per_sm)) * sms, (npx + 7) / 8));
    *nsplit = grid;
    CNNCRF_TRY(train_zero_border(out, nimg, H, W, 128, p, q, st));
    {
        CNNCRF_PROF("l2norm_bwd", st);
        k_l2norm_tanh_bwd_pad<<<grid, 256, 0, st>>>((const __nv_bfloat16 *)y, ys, df, H, W, C, npx, p, q,
                                                    (__nv_bfloat16 *)out, part);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

template <class T>
static int corr_bwd_t(const T *fl, const T *fr, int fs, const float *gvol, const float *d_list, int npairs, int H,
                      int W, int C, int D, int omin, int omax, float *dfl, float *dfr, cudaStream_t st)
{
    if (C > 128) return fail(CNNCRF_EINVAL, "corr_bwd: %d channels > 128", C);
    int dev = 0, maxsm = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    {
        // the blocked kernel (integer lists have distinct offsets: the stored list strictly decreases)
        const int band = omax - omin + 1, Cs = (C + 3) & ~3;
        const size_t sm = corr_bwd_blk_smem(band, Cs, sizeof(T), D);
        if (sm <= (size_t)maxsm) {
            CNNCRF_CUDA(cudaFuncSetAttribute(k_corr_bwd_blk<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            const dim3 g(ceil_div(W, CB_TX), H, npairs);
            {
                CNNCRF_PROF("corr_bwd", st);
                k_corr_bwd_blk<T><<<g, 256, sm, st>>>(fr, fs, gvol, d_list, H, W, C, Cs, D, 0, omin, band, dfl);
                k_corr_bwd_blk<T><<<g, 256, sm, st>>>(fl, fs, gvol, d_list, H, W, C, Cs, D, 1, -omax, band, dfr);
            }
            CNNCRF_CHECK_LAUNCH();
            return CNNCRF_OK;
        }
    }
    const int span = 32 + omax - omin;
    const size_t smem = sizeof(float) * (size_t)span * C + sizeof(int) * (size_t)D;
    if (smem > 227 * 1024) return fail(CNNCRF_EUNSUPPORTED, "corr_bwd: band %d too wide", omax - omin);
    CNNCRF_CUDA(cudaFuncSetAttribute(k_corr_bwd_left<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CNNCRF_CUDA(cudaFuncSetAttribute(k_corr_bwd_right<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const dim3 g(ceil_div(W, 32), H, npairs);
    {
        CNNCRF_PROF("corr_bwd", st);
        k_corr_bwd_left<T><<<g, 128, smem, st>>>(fr, fs, gvol, d_list, H, W, C, D, omin, span, dfl);
        k_corr_bwd_right<T><<<g, 128, smem, st>>>(fl, fs, gvol, d_list, H, W, C, D, omax, span, dfr);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_corr_bwd(const void *fl, const void *fr, bool bf16, int fs, const float *gvol, const float *d_list,
                   int npairs, int H, int W, int C, int D, int omin, int omax, float *dfl, float *dfr, cudaStream_t st)
{
    if (bf16)
        return corr_bwd_t((const __nv_bfloat16 *)fl, (const __nv_bfloat16 *)fr, fs, gvol, d_list, npairs, H, W, C, D,
                          omin, omax, dfl, dfr, st);
    return corr_bwd_t((const float *)fl, (const float *)fr, fs, gvol, d_list, npairs, H, W, C, D, omin, omax, dfl, dfr,
                      st);
}

int train_wgrad_splits(long P)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        sms = 148;
    return (int)std::max(1L, std::min((long)4 * sms, P / 256));
}

int train_wgrad_splits_k(long P, int K)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                  cudaSuccess)
        sms = 148;
    const long kt = ceil_div(K, WG_KT);
    long ns = std::max(1L, 4L * sms / kt);
    ns = std::min(ns, std::max(1L, P / 512));
    return (int)std::min(ns, 1024L);
}

template <class T>
static int wgrad_t(const float *dz, int Cout, const T *in, long in_pix, long in_row, long in_img, int Cin, int kh,
                   int kw, int nimg, int Ho, int Wo, float *part, float *dw, float *db, float *partb, cudaStream_t st)
{
    if (Cout > 128) return fail(CNNCRF_EINVAL, "wgrad: %d output channels > 128", Cout);
    WgradArgs<T> a;
    a.dz = dz, a.Cout = Cout, a.in = in, a.in_pix = in_pix, a.in_row = in_row, a.in_img = in_img;
    a.Cin = Cin, a.kh = kh, a.kw = kw, a.Ho = Ho, a.Wo = Wo;
    a.P = (long)nimg * Ho * Wo;
    const int K = kh * kw * Cin;
    const int ns = train_wgrad_splits_k(a.P, K);
    a.chunk = (a.P + ns - 1) / ns;
    a.part = part;
    {
        CNNCRF_PROF("wgrad", st);
        k_wgrad<T><<<dim3(ceil_div(K, WG_KT), ns), 256, 0, st>>>(a);
        k_wgrad_reduce<<<ceil_div((long)Cout * K, 32), 256, 0, st>>>(part, ns, Cout, Cin, kh, kw, dw);
    }
    if (db) CNNCRF_TRY(train_bias_grad(dz, Cout, a.P, partb, db, st));
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_wgrad(const float *dz, int Cout, const void *in, bool bf16, long in_pix, long in_row, long in_img, int Cin,
                int kh, int kw, int nimg, int Ho, int Wo, float *part, float *dw, float *db, float *partb, cudaStream_t st)
{
    if (bf16)
        return wgrad_t(dz, Cout, (const __nv_bfloat16 *)in, in_pix, in_row, in_img, Cin, kh, kw, nimg, Ho, Wo, part,
                       dw, db, partb, st);
    return wgrad_t(dz, Cout, (const float *)in, in_pix, in_row, in_img, Cin, kh, kw, nimg, Ho, Wo, part, dw, db, partb,
                   st);
}

int train_bias_grad(const float *dz, int Cout, long P, float *partb, float *db, cudaStream_t st)
{
    const int ns = train_wgrad_splits(P);
    const long chunk = (P + ns - 1) / ns;
    if (Cout > 128) return fail(CNNCRF_EINVAL, "bias grad: %d channels > 128", Cout);
    k_bias_part<<<ns, dim3(128, 4), 0, st>>>(dz, Cout, P, chunk, partb);
    k_bias_reduce<<<ceil_div(Cout, 32), 256, 0, st>>>(partb, ns, Cout, db);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_to_bf16_c64(const float *in, long npx, int C, void *out, cudaStream_t st)
{
    if (C > 64 || ((uintptr_t)out & 15)) return fail(CNNCRF_EINVAL, "to_bf16_c64: %d channels", C);
    k_to_bf16_c64<<<ceil_div(npx * 8, 256), 256, 0, st>>>(in, npx, C, (__nv_bfloat16 *)out);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_wgrad_head(const float *gh, const void *y, bool bf16, int ys, long P, int C, float *part, float *dw,
                     cudaStream_t st)
{
    if (C > 128) return fail(CNNCRF_EINVAL, "head wgrad: %d channels > 128", C);
    const int ns = train_wgrad_splits(P);
    const long chunk = (P + ns - 1) / ns;
    {
        CNNCRF_PROF("wgrad", st);
        const dim3 blk(128, 2, 2);
        if (bf16)
            k_wgrad_head<<<ns, blk, 0, st>>>(gh, (const __nv_bfloat16 *)y, ys, P, chunk, C, part);
        else
            k_wgrad_head<<<ns, blk, 0, st>>>(gh, (const float *)y, ys, P, chunk, C, part);
        // the 2 x C sums, flat: the npz layout w[o][c][1][1]
        k_bias_reduce<<<ceil_div(2 * C, 32), 256, 0, st>>>(part, ns, 2 * C, dw);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_bias_reduce(const float *part, int nsplit, int Cout, float *db, cudaStream_t st)
{
    k_bias_reduce<<<ceil_div(Cout, 32), 256, 0, st>>>(part, nsplit, Cout, db);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_head_bwd(const void *y2, bool bf16, int ys, const float *wh, const float *gpw, int nimg, int npx, int P,
                   float *gh, float *dy2, cudaStream_t st)
{
    const dim3 g(ceil_div(npx, 128), nimg);
    if (bf16)
        k_head_bwd<<<g, 128, 0, st>>>((const __nv_bfloat16 *)y2, ys, wh, gpw, npx, P, gh, dy2);
    else
        k_head_bwd<<<g, 128, 0, st>>>((const float *)y2, ys, wh, gpw, npx, P, gh, dy2);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_head_tanh_bwd_pad(const void *y2, int ys, const float *wh, const float *gpw, int nimg, int H, int W, int P,
                            int p, int q, float *gh, void *out, float *part, int *nsplit, cudaStream_t st)
{
    if (P > 64 || P % 2 || ys % 2 || ((uintptr_t)out & 15) || ((uintptr_t)y2 & 3) || ((uintptr_t)gh & 7) ||
        (long)nimg * H * W >= (1L << 31))
        return fail(CNNCRF_EINVAL, "head_tanh_bwd_pad: %d channels / layout", P);
    int dev = 0, sms = 0, per_sm = 1;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CNNCRF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_head_tanh_bwd_pad, 256, 0));
    const long npx = (long)nimg * H * W;
    const int grid = (int)std::max(1L, std::min((long)std::min(4, std::max(1, per_sm)) * sms, (npx + 7) / 8));
    *nsplit = grid;
    CNNCRF_TRY(train_zero_border(out, nimg, H, W, 64, p, q, st));
    k_head_tanh_bwd_pad<<<grid, 256, 0, st>>>((const __nv_bfloat16 *)y2, ys, wh, gpw, H, W, P, npx, p, q, gh,
                                              (__nv_bfloat16 *)out, part);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_augment(const float *vol, const int32_t *gt, long npx, int D, float *aug, int *err, cudaStream_t st)
{
    if (((uintptr_t)vol & 15) || ((uintptr_t)aug & 15)) return fail(CNNCRF_EINVAL, "augment: alignment");
    int dev = 0, sms = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    k_augment<<<(int)std::min((npx + 7) / 8, (long)8 * sms), 256, 0, st>>>(vol, gt, npx, D, aug, err);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_hinge(const float *vol, const float *w, const int32_t *gt, const int32_t *yh, int npairs, int W, int H,
                int D, float lam, const float rho[9], float L2, int delta, float gscale, float *gvol, float *gpw,
                double *contrib, double *rows, cudaStream_t st)
{
    HingeArgs a;
    a.gscale = gscale;
    a.vol = vol, a.w = w, a.gt = gt, a.yh = yh, a.W = W, a.H = H, a.D = D, a.lam = lam, a.L2 = L2, a.delta = delta;
    for (int t = 0; t < 9; ++t) a.rho[t] = rho[t];
    a.gvol = gvol, a.gpw = gpw, a.contrib = contrib;
    k_hinge<<<dim3(ceil_div(W, 128), H, npairs), 128, 0, st>>>(a);
    k_row_sums_d<<<ceil_div((long)npairs * H, 128), 128, 0, st>>>(contrib, (long)npairs * H, W, rows);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

int train_sgd(float *theta, const float *g, float *v, long n, float lr, float mu, cudaStream_t st)
{
    k_sgd<<<ceil_div(n, 256), 256, 0, st>>>(theta, g, v, n, lr, mu);
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
