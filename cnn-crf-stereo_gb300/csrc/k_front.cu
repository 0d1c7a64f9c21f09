// k_front.cu -- mirror padding and RGB normalisation (the front end of
// ColorStereoNet::predict).  Compiled with --fmad=false: results must match
// the CPU oracle bit for bit.
#include "common.h"
#include "kernels.h"

namespace cnncrf {
namespace k {

namespace {

// cudaAddressModeMirror at texel centres (stereo/stereo.cu:879-911): symmetric
// reflection, edge sample repeated, period 2n.
__device__ __forceinline__ int mirror_idx(int i, int n)
{
    int m = i % (2 * n);
    if (m < 0) m += 2 * n;
    return m >= n ? 2 * n - 1 - m : m;
}

__global__ void k_pad(const float4 *__restrict__ in, int W, int H, int p, float4 *__restrict__ out)
{
    int Wp = W + 2 * p, Hp = H + 2 * p;
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)Wp * Hp) return;
    in += (long)blockIdx.y * W * H; // image of the batch
    out += (long)blockIdx.y * Wp * Hp;
    int y = (int)(i / Wp), x = (int)(i - (long)y * Wp);
    out[i] = in[(long)mirror_idx(y - p, H) * W + mirror_idx(x - p, W)];
}

// value of plane c at pixel i: RGB channel, or rgb_to_gray_kernel's weights
// (stereo/stereo.cu:853-863) evaluated in double and rounded once.
__device__ __forceinline__ float plane_val(const float *rgba, long i, int c, int gray)
{
    const float *px = rgba + 4 * i;
    if (gray)
        return (float)(0.2989 * (double)px[0] + 0.5870 * (double)px[1] + 0.1140 * (double)px[2]);
    return px[c];
}

// FP64 sums in a fixed order shared with the CPU oracle: lane j of a warp sums
// the elements j, j+32, j+64, ... in ascending order, then the 32 partial sums
// are combined by an xor butterfly (offsets 16, 8, 4, 2, 1).
__device__ __forceinline__ double warp_tree_sum(double s)
{
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) s = s + __shfl_xor_sync(0xffffffffu, s, off);
    return s;
}

// One warp per (plane, row).  pass 0 sums the values, pass 1 the squares of
// (v - mean_c) rounded to float.
__global__ void k_rowsums(const float *__restrict__ rgba, int Wp, int Hp, int planes, int gray,
                          int pass, const float *__restrict__ stats, double *__restrict__ rows)
{
    const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (w >= planes * Hp) return;
    rgba += (long)blockIdx.y * Wp * Hp * 4; // image of the batch
    rows += (long)blockIdx.y * 3 * Hp;
    stats += blockIdx.y * 8;
    const int c = w / Hp, y = w - c * Hp;
    const long base = (long)y * Wp;
    double s = 0.0;
    if (pass == 0) {
        for (int x = lane; x < Wp; x += 32) s += (double)plane_val(rgba, base + x, c, gray);
    } else {
        const float mean = stats[c];
        for (int x = lane; x < Wp; x += 32) {
            const float v = __fsub_rn(plane_val(rgba, base + x, c, gray), mean);
            s += (double)__fmul_rn(v, v);
        }
    }
    s = warp_tree_sum(s);
    if (lane == 0) rows[w] = s;
}

// One warp per plane: the row sums in the same lane / butterfly order -> mean
// (pass 0) or population std (pass 1).
__global__ void k_finalize(const double *__restrict__ rows, int Hp, int planes, long N, int pass,
                           float *__restrict__ stats)
{
    const int c = blockIdx.x, lane = threadIdx.x;
    rows += (long)blockIdx.y * 3 * Hp;
    stats += blockIdx.y * 8;
    double s = 0.0;
    for (int y = lane; y < Hp; y += 32) s += rows[c * Hp + y];
    s = warp_tree_sum(s);
    if (lane == 0) {
        if (pass == 0) stats[c] = (float)(s / (double)N);
        else stats[4 + c] = (float)sqrt(s / (double)N);
    }
}

__global__ void k_norm_write(const float *__restrict__ rgba, int Wp, int Hp, int ic,
                             const float *__restrict__ stats, float *__restrict__ out)
{
    long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (long)Wp * Hp) return;
    rgba += (long)blockIdx.y * Wp * Hp * 4;
    stats += blockIdx.y * 8;
    out += (long)blockIdx.y * Wp * Hp * ic;
    int gray = ic == 1;
    int planes = gray ? 1 : 3;
    for (int c = 0; c < planes; ++c) {
        float v = __fsub_rn(plane_val(rgba, i, c, gray), stats[c]);
        float sd = stats[4 + c];
        out[i * ic + c] = sd > 0.0f ? __fdiv_rn(v, sd) : 0.0f;
    }
    if (ic == 5) { // stereo/colorstereonet.cpp:102-121
        int y = (int)(i / Wp), x = (int)(i - (long)y * Wp);
        out[i * ic + 3] = (float)(((double)x - (double)Wp / 2.0) / (double)Wp);
        out[i * ic + 4] = (float)(((double)y - (double)Hp / 2.0) / (double)Hp);
    }
}

} // namespace

int pad_rgba(const float *in, int W, int H, int p, float *out, cudaStream_t st, int nimg)
{
    long n = (long)(W + 2 * p) * (H + 2 * p);
    {
        CNNCRF_PROF("pad", st);
        k_pad<<<dim3(ceil_div(n, 256), nimg), 256, 0, st>>>((const float4 *)in, W, H, p, (float4 *)out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

size_t normalize_scratch_bytes(int Hp, int nimg) { return (sizeof(double) * 3 * (size_t)Hp + 32) * nimg + 64; }

int normalize(const float *rgba, int Wp, int Hp, int ic, float *out, void *scratch, cudaStream_t st, int nimg)
{
    int gray = ic == 1, planes = gray ? 1 : 3;
    double *rows = (double *)scratch;
    float *stats = (float *)((char *)scratch + sizeof(double) * 3 * (size_t)Hp * nimg);
    long N = (long)Wp * Hp;
    const long nthreads = 32L * planes * Hp;
    {
        CNNCRF_PROF("rowsums", st);
        k_rowsums<<<dim3(ceil_div(nthreads, 256), nimg), 256, 0, st>>>(rgba, Wp, Hp, planes, gray, 0, stats, rows);
    }
    {
        CNNCRF_PROF("finalize", st);
        k_finalize<<<dim3(planes, nimg), 32, 0, st>>>(rows, Hp, planes, N, 0, stats);
    }
    {
        CNNCRF_PROF("rowsums", st);
        k_rowsums<<<dim3(ceil_div(nthreads, 256), nimg), 256, 0, st>>>(rgba, Wp, Hp, planes, gray, 1, stats, rows);
    }
    {
        CNNCRF_PROF("finalize", st);
        k_finalize<<<dim3(planes, nimg), 32, 0, st>>>(rows, Hp, planes, N, 1, stats);
    }
    {
        CNNCRF_PROF("norm_write", st);
        k_norm_write<<<dim3(ceil_div(N, 256), nimg), 256, 0, st>>>(rgba, Wp, Hp, ic, stats, out);
    }
    CNNCRF_CHECK_LAUNCH();
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
