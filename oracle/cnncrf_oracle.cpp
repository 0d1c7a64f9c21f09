// cnncrf_oracle.cpp -- TEST INFRASTRUCTURE (see cnncrf_oracle.h): the CPU
// restatement of the reference hot path that tests, smoke() and bench.py's
// CPU legs check against.  Never linked into libcnncrf.so.
//
// Each function cites the reference file:line it restates.  Arithmetic order
// is spelled out (explicit fmaf, left-to-right adds) because the float build
// is compared bit for bit with the GPU FP32 path.
#include "cnncrf_oracle.h"

#include "../include/cnncrf_fmath.h"
#include "../include/cnncrf_xavier.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class T> inline T fmaT(T a, T b, T c);
template <> inline float fmaT<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <> inline double fmaT<double>(double a, double b, double c) { return std::fma(a, b, c); }
template <class T> inline T tanhT(T x);
template <> inline float tanhT<float>(float x) { return cnncrf_tanhf(x); }
template <> inline double tanhT<double>(double x) { return std::tanh(x); }
template <class T> inline T expT(T x);
template <> inline float expT<float>(float x) { return cnncrf_expf(x); }
template <> inline double expT<double>(double x) { return std::exp(x); }

inline float fmin2(float a, float b) { return b < a ? b : a; }

struct Layer {
    int cin, cout, kh, kw, act, wslot, bslot;
};

// ConcatStereoNet's growth rate per depth (stereo/concatstereonet.cpp:28-56); 0: no such net
int growth_rate(int layers)
{
    switch (layers) {
    case 3: return 33;
    case 5: return 20;
    case 7: return 14;
    case 10: return 10;
    case 15: return 7;
    case 20: return 5;
    case 25: return 4;
    case 33: return 3;
    case 50: return 2;
    case 100: return 1;
    default: return 0;
    }
}

// channels of the features the correlation reads
int feature_width(const oracle_cfg *c)
{
    return c->topology == 2 ? growth_rate(c->num_layers) * c->num_layers : c->feat_channels;
}

// stereo/stereonet.cpp:69-133 (feature net), 159-167 (pairwise net);
// topology 2: ConcatStereoNet (stereo/concatstereonet.cpp:72-127), every layer
// a 3x3 conv with zero padding 1 to the growth rate g, fed the previous
// layer's output; the features are all L layer outputs side by side (g L
// channels, layer 1 first)
std::vector<Layer> feature_layers(const oracle_cfg *c)
{
    std::vector<Layer> v;
    if (c->topology == 2) {
        int g = growth_rate(c->num_layers);
        v.push_back({c->in_channels, g, 3, 3, 1, 0, 1});
        for (int l = 1; l < c->num_layers; ++l) v.push_back({g, g, 3, 3, 1, 2 * l, 2 * l + 1});
        return v;
    }
    int F = c->feat_channels;
    v.push_back({c->in_channels, F, 3, 3, 1, 0, 1});
    int k = c->topology == 0 ? 2 : 3;
    for (int l = 1; l < c->num_layers; ++l) v.push_back({F, F, k, k, 1, 2 * l, 2 * l + 1});
    return v;
}

std::vector<Layer> pairwise_layers(const oracle_cfg *c)
{
    std::vector<Layer> v;
    if (c->topology == 2) { // a 3x3 conv of the features to 2 channels, zero padding 1, no bias, |tanh|
        v.push_back({feature_width(c), 2, 3, 3, 3, 2 * c->num_layers, -1});
        return v;
    }
    int base = 2 * c->num_layers;
    int pc = c->in_channels == 1 ? 1 : 3;
    int P = c->pw_channels;
    v.push_back({pc, P, 3, 3, 1, base, base + 1});
    v.push_back({P, P, 3, 3, 1, base + 2, base + 3});
    v.push_back({P, 2, 1, 1, 2, base + 4, -1});
    return v;
}

void set_threads(int t)
{
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

// ---------------------------------------------------------------- normalise
// stereo/colorstereonet.cpp:53-64 (+ xy 102-121), stereo/utils.cu:169-237.
// Sums are FP64 in a fixed order (the reference's thrust reduction order is
// unspecified): 32 partial sums, partial j taking elements j, j+32, ... in
// ascending order, combined by an xor butterfly 16, 8, 4, 2, 1 -- first per
// row, then over the row sums.
double tree_sum_strided(const double *v, long n)
{
    double s[32] = {0}, t[32];
    for (long i = 0; i < n; ++i) s[i % 32] += v[i];
    for (int off = 16; off >= 1; off >>= 1) {
        for (int j = 0; j < 32; ++j) t[j] = s[j] + s[j ^ off];
        std::memcpy(s, t, sizeof s);
    }
    return s[0];
}

template <class T>
void normalize_T(const float *rgba, int Wp, int Hp, int ic, T *out)
{
    long N = (long)Wp * Hp;
    int planes = ic == 1 ? 1 : 3;
    std::vector<T> pl((size_t)N);
    std::vector<double> rs((size_t)Hp);
    for (int c = 0; c < planes; ++c) {
        for (long i = 0; i < N; ++i) {
            const float *px = rgba + 4 * i;
            if (ic == 1) // stereo/stereo.cu:853-863
                pl[i] = (T)(float)(0.2989 * (double)px[0] + 0.5870 * (double)px[1] +
                                   0.1140 * (double)px[2]);
            else
                pl[i] = (T)px[c];
        }
        std::vector<double> row((size_t)Wp);
        for (int y = 0; y < Hp; ++y) {
            for (int x = 0; x < Wp; ++x) row[x] = (double)pl[(long)y * Wp + x];
            rs[y] = tree_sum_strided(row.data(), Wp);
        }
        double tot = tree_sum_strided(rs.data(), Hp);
        T mean = (T)(tot / (double)N);
        for (long i = 0; i < N; ++i) pl[i] = pl[i] - mean;
        for (int y = 0; y < Hp; ++y) {
            for (int x = 0; x < Wp; ++x) {
                T v = pl[(long)y * Wp + x];
                T sq = v * v;
                row[x] = (double)sq;
            }
            rs[y] = tree_sum_strided(row.data(), Wp);
        }
        tot = tree_sum_strided(rs.data(), Hp);
        T sd = (T)std::sqrt(tot / (double)N);
        for (long i = 0; i < N; ++i) out[i * ic + c] = sd > (T)0 ? pl[i] / sd : (T)0;
    }
    if (ic == 5) {
        for (int y = 0; y < Hp; ++y)
            for (int x = 0; x < Wp; ++x) {
                long i = (long)y * Wp + x;
                out[i * ic + 3] = (T)(float)(((double)x - (double)Wp / 2.0) / (double)Wp);
                out[i * ic + 4] = (T)(float)(((double)y - (double)Hp / 2.0) / (double)Hp);
            }
    }
}

// ---------------------------------------------------------------- conv
// stereo/operators/convolution.cpp:104-108,141-152 (CUDNN_CONVOLUTION: flipped
// kernel, valid, stride 1), bias.cpp:58-67 (y += b), activation.cpp:33-41.
// Sum order per output: ky, kx, ci ascending, acc = fma(w, x, acc) from 0.
template <class T>
void conv_T(const T *in, int H, int W, int Cin, const float *w, const float *b, int Cout, int kh,
            int kw, int act, T *out)
{
    int Ho = H - kh + 1, Wo = W - kw + 1;
    int K = kh * kw * Cin;
    std::vector<T> Wt((size_t)K * Cout);
    for (int co = 0; co < Cout; ++co)
        for (int ci = 0; ci < Cin; ++ci)
            for (int ky = 0; ky < kh; ++ky)
                for (int kx = 0; kx < kw; ++kx) {
                    int k = (ky * kw + kx) * Cin + ci;
                    Wt[(size_t)k * Cout + co] =
                        (T)w[(((size_t)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)];
                }
#pragma omp parallel for schedule(dynamic, 1)
    for (int oy = 0; oy < Ho; ++oy) {
        std::vector<T> acc((size_t)Cout);
        for (int ox = 0; ox < Wo; ++ox) {
            std::fill(acc.begin(), acc.end(), (T)0);
            for (int ky = 0; ky < kh; ++ky)
                for (int kx = 0; kx < kw; ++kx) {
                    const T *src = in + ((size_t)(oy + ky) * W + ox + kx) * Cin;
                    const T *wk = Wt.data() + (size_t)((ky * kw + kx) * Cin) * Cout;
                    for (int ci = 0; ci < Cin; ++ci) {
                        T xv = src[ci];
                        const T *wr = wk + (size_t)ci * Cout;
                        T *a = acc.data();
                        for (int co = 0; co < Cout; ++co) a[co] = fmaT<T>(wr[co], xv, a[co]);
                    }
                }
            T *dst = out + ((size_t)oy * Wo + ox) * Cout;
            for (int co = 0; co < Cout; ++co) {
                T v = acc[co];
                if (b) v = v + (T)b[co];
                if (act == 1) v = tanhT<T>(v);
                else if (act == 2) v = std::fabs(v);
                else if (act == 3) v = std::fabs(tanhT<T>(v));
                dst[co] = v;
            }
        }
    }
}

template <class T> void l2norm_T(T *f, long npx, int C)
{
#pragma omp parallel for
    for (long i = 0; i < npx; ++i) {
        T *p = f + i * C;
        T s = 0;
        for (int c = 0; c < C; ++c) s = fmaT<T>(p[c], p[c], s);
        T n = std::sqrt(s);
        for (int c = 0; c < C; ++c) p[c] = n > (T)0 ? p[c] / n : (T)0;
    }
}

// ---------------------------------------------------------------- correlation
// stereo/operators/stereocorrelation.cu:66-142 (NHWC kernels, rectCorr = 0) and
// the dispatch at :364-373,394-400.  Out-of-image taps (w + d < 0) give 0.
// Where the reference would read past the right edge (w + d > W-1) the index
// is clamped / the tap gives 0 instead.
template <class T>
void correlation_T(const T *fl, const T *fr, int H, int W, int C, const float *list, int D,
                   int force_interp, T *out)
{
    bool isf = force_interp || oracle_disp_is_float(list, D);
#pragma omp parallel for
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const T *a = fl + ((size_t)y * W + x) * C;
            T *o = out + ((size_t)y * W + x) * D;
            for (int k = 0; k < D; ++k) {
                float s = list[k];
                float w2 = (float)x + s;
                T acc = 0;
                if (!isf) {
                    if (w2 >= 0.0f) {
                        int xs = x + (int)s;
                        if (xs <= W - 1) {
                            const T *bb = fr + ((size_t)y * W + xs) * C;
                            for (int c = 0; c < C; ++c) acc = fmaT<T>(a[c], bb[c], acc);
                        }
                    }
                } else if (w2 >= 0.0f) {
                    int x0 = (int)floorf(w2);
                    int x1 = (int)(w2 + 1.0f);
                    int x0c = std::min(x0, W - 1), x1c = std::min(x1, W - 1);
                    T num = (T)w2 - (T)(float)x0;
                    T den = (T)(float)x1 - (T)(float)x0;
                    const T *b0 = fr + ((size_t)y * W + x0c) * C;
                    const T *b1 = fr + ((size_t)y * W + x1c) * C;
                    for (int c = 0; c < C; ++c) {
                        T y0 = b0[c], y1 = b1[c];
                        T it = y0 + ((y1 - y0) * num) / den;
                        acc = fmaT<T>(a[c], it, acc);
                    }
                }
                o[k] = acc;
            }
        }
}

// stereo/operators/softmax.cpp:30-38 (channel softmax over D) + stereo/utils.cu:289-292
// (negate).  The FP32 sum follows the warp layout of the GPU kernel: lane j
// owns k = j + 32r, sums its values left to right, then xor-butterfly 16..1.
float tree_sum32(const float *e, int D)
{
    float s[32], t[32];
    for (int j = 0; j < 32; ++j) {
        s[j] = j < D ? e[j] : 0.0f;
        for (int k = j + 32; k < ((D + 31) / 32) * 32; k += 32) s[j] = s[j] + (k < D ? e[k] : 0.0f);
    }
    for (int off = 16; off >= 1; off >>= 1) {
        for (int j = 0; j < 32; ++j) t[j] = s[j] + s[j ^ off];
        std::memcpy(s, t, sizeof s);
    }
    return s[0];
}

template <class T> void unary_T(T *vol, long npx, int D, int unary);
template <> void unary_T<float>(float *vol, long npx, int D, int unary)
{
#pragma omp parallel for
    for (long i = 0; i < npx; ++i) {
        float *v = vol + i * D;
        if (unary == 1) {
            for (int k = 0; k < D; ++k) v[k] = 1.0f - v[k];
            continue;
        }
        float m = -FLT_MAX;
        for (int k = 0; k < D; ++k) m = std::max(m, v[k]);
        std::vector<float> e((size_t)D);
        for (int k = 0; k < D; ++k) e[k] = cnncrf_expf(v[k] - m);
        float S = tree_sum32(e.data(), D);
        for (int k = 0; k < D; ++k) v[k] = -(e[k] / S);
    }
}
template <> void unary_T<double>(double *vol, long npx, int D, int unary)
{
#pragma omp parallel for
    for (long i = 0; i < npx; ++i) {
        double *v = vol + i * D;
        if (unary == 1) {
            for (int k = 0; k < D; ++k) v[k] = 1.0 - v[k];
            continue;
        }
        double m = -DBL_MAX;
        for (int k = 0; k < D; ++k) m = std::max(m, v[k]);
        double S = 0;
        for (int k = 0; k < D; ++k) S += std::exp(v[k] - m);
        for (int k = 0; k < D; ++k) v[k] = -(std::exp(v[k] - m) / S);
    }
}

// ---------------------------------------------------------------- predict
// ColorStereoNet::predict (stereo/colorstereonet.cpp:38-133) +
// StereoNet::performPrediction (stereo/stereonet.cpp:250-421).
// [H][W][C] -> [H+2][W+2][C] with a zero border (a 3x3 conv with zero padding 1
// is the valid conv of this)
template <class T> std::vector<T> zero_border(const T *src, int H, int W, int C)
{
    std::vector<T> o((size_t)(H + 2) * (W + 2) * C, (T)0);
    for (int y = 0; y < H; ++y)
        std::memcpy(&o[((size_t)(y + 1) * (W + 2) + 1) * C], src + (size_t)y * W * C, sizeof(T) * (size_t)W * C);
    return o;
}

// ConcatStereoNet::initNet + ColorStereoNet::predict (stereo/concatstereonet.cpp:72-127,
// stereo/colorstereonet.cpp:38-77) as this library builds the net: no mirror
// padding (stereo/stereo.cpp:214-216 sets it to 0), every conv zero-padded,
// the correlation over all g L feature channels, and the pairwise weights
// |tanh(conv3x3(features))| from the raw (not normalised) left features.
template <class T>
int predict_concat_T(const oracle_cfg *cfg, const float *const *params, const float *lp, const float *rp,
                     int w, int h, const float *list, int D, int force_interp, T *vol, T *pw)
{
    const int H = h, W = w, ic = cfg->in_channels;
    const int g = growth_rate(cfg->num_layers), C = feature_width(cfg);
    if (g == 0) return 3;
    auto layers = feature_layers(cfg);
    std::vector<T> feat[2];
    const float *img[2] = {lp, rp};
    for (int s = 0; s < 2; ++s) {
        std::vector<T> n((size_t)W * H * ic), t((size_t)W * H * g);
        normalize_T<T>(img[s], w, h, ic, n.data());
        feat[s].assign((size_t)W * H * C, (T)0);
        std::vector<T> cur = zero_border<T>(n.data(), H, W, ic);
        for (size_t l = 0; l < layers.size(); ++l) {
            const Layer &L = layers[l];
            conv_T<T>(cur.data(), H + 2, W + 2, L.cin, params[L.wslot], params[L.bslot], g, 3, 3, L.act, t.data());
            for (long i = 0; i < (long)H * W; ++i)
                for (int c = 0; c < g; ++c) feat[s][(size_t)i * C + l * g + c] = t[(size_t)i * g + c];
            cur = zero_border<T>(t.data(), H, W, g);
        }
    }
    if (cfg->with_pairwise && pw) {
        const Layer P = pairwise_layers(cfg)[0];
        std::vector<T> z = zero_border<T>(feat[0].data(), H, W, C), t((size_t)W * H * 2);
        conv_T<T>(z.data(), H + 2, W + 2, C, params[P.wslot], nullptr, 2, 3, 3, P.act, t.data());
        for (long i = 0; i < (long)H * W; ++i) {
            pw[i] = t[(size_t)i * 2];
            pw[(size_t)H * W + i] = t[(size_t)i * 2 + 1];
        }
    }
    if (cfg->unary == 1) {
        l2norm_T<T>(feat[0].data(), (long)H * W, C);
        l2norm_T<T>(feat[1].data(), (long)H * W, C);
    }
    correlation_T<T>(feat[0].data(), feat[1].data(), H, W, C, list, D, force_interp, vol);
    unary_T<T>(vol, (long)H * W, D, cfg->unary);
    return 0;
}

template <class T>
int predict_T(const oracle_cfg *cfg, const float *const *params, const float *lp, const float *rp,
              int w, int h, const float *list, int D, int force_interp, T *vol, T *pw)
{
    if (cfg->topology == 2) return predict_concat_T<T>(cfg, params, lp, rp, w, h, list, D, force_interp, vol, pw);
    int p = oracle_padding(cfg);
    if (p < 0) return 1;
    int H = h - 2 * p, W = w - 2 * p;
    int ic = cfg->in_channels;
    std::vector<T> nl((size_t)w * h * ic), nr((size_t)w * h * ic);
    normalize_T<T>(lp, w, h, ic, nl.data());
    normalize_T<T>(rp, w, h, ic, nr.data());
    auto layers = feature_layers(cfg);
    std::vector<T> a = nl, b = nr, t;
    int ch = h, cw = w;
    for (auto &L : layers) {
        int oh = ch - L.kh + 1, ow = cw - L.kw + 1;
        t.assign((size_t)oh * ow * L.cout, (T)0);
        conv_T<T>(a.data(), ch, cw, L.cin, params[L.wslot], L.bslot >= 0 ? params[L.bslot] : nullptr,
                  L.cout, L.kh, L.kw, L.act, t.data());
        a.swap(t);
        t.assign((size_t)oh * ow * L.cout, (T)0);
        conv_T<T>(b.data(), ch, cw, L.cin, params[L.wslot], L.bslot >= 0 ? params[L.bslot] : nullptr,
                  L.cout, L.kh, L.kw, L.act, t.data());
        b.swap(t);
        ch = oh;
        cw = ow;
    }
    if (ch != H || cw != W) return 2;
    int C = cfg->feat_channels;
    if (cfg->unary == 1) {
        l2norm_T<T>(a.data(), (long)H * W, C);
        l2norm_T<T>(b.data(), (long)H * W, C);
    }
    correlation_T<T>(a.data(), b.data(), H, W, C, list, D, force_interp, vol);
    unary_T<T>(vol, (long)H * W, D, cfg->unary);
    if (cfg->with_pairwise && pw) {
        int cr = p - 2;
        int pc = ic == 1 ? 1 : 3;
        int ph = H + 4, pww = W + 4;
        std::vector<T> pin((size_t)ph * pww * pc);
        for (int y = 0; y < ph; ++y)
            for (int x = 0; x < pww; ++x)
                for (int c = 0; c < pc; ++c)
                    pin[((size_t)y * pww + x) * pc + c] = nl[((size_t)(y + cr) * w + x + cr) * ic + c];
        auto pl = pairwise_layers(cfg);
        std::vector<T> cur = pin;
        int hh = ph, ww = pww;
        for (auto &L : pl) {
            int oh = hh - L.kh + 1, ow = ww - L.kw + 1;
            t.assign((size_t)oh * ow * L.cout, (T)0);
            conv_T<T>(cur.data(), hh, ww, L.cin, params[L.wslot],
                      L.bslot >= 0 ? params[L.bslot] : nullptr, L.cout, L.kh, L.kw, L.act, t.data());
            cur.swap(t);
            hh = oh;
            ww = ow;
        }
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                pw[(size_t)y * W + x] = cur[((size_t)y * W + x) * 2 + 0];
                pw[(size_t)H * W + (size_t)y * W + x] = cur[((size_t)y * W + x) * 2 + 1];
            }
    }
    return 0;
}

// ---------------------------------------------------------------- CRF
// Our SlackProp spec (the library is absent; call sites stereo/stereo.cpp:140-154).
struct Rho {
    int delta;
    float rho[9];
    float L2;
};

Rho make_rho(float L1, float L2, int delta, int shape)
{
    Rho r;
    r.delta = delta;
    r.L2 = L2;
    r.rho[0] = 0.0f;
    for (int t = 1; t <= delta; ++t) r.rho[t] = shape == 0 ? fmin2(L1, L2) : fmin2(L1 * (float)t, L2);
    return r;
}

// out_k = min(v_k, v_{k+-t} + w*rho_t, g + w*L2) - g,  g = min v
void minconv(const float *v, float g, float w, const Rho &r, int D, float *out)
{
    float c[9];
    for (int t = 1; t <= r.delta; ++t) c[t] = w * r.rho[t];
    float base = g + w * r.L2;
    for (int k = 0; k < D; ++k) {
        float o = v[k];
        for (int t = 1; t <= r.delta; ++t) {
            if (k - t >= 0) o = fmin2(o, v[k - t] + c[t]);
            if (k + t < D) o = fmin2(o, v[k + t] + c[t]);
        }
        o = fmin2(o, base);
        out[k] = o - g;
    }
}

inline float vmin(const float *v, int D)
{
    float m = v[0];
    for (int k = 1; k < D; ++k) m = fmin2(m, v[k]);
    return m;
}

// One chain.  unary(i, k) reads the subproblem's unary; on the backward pass
// the slack fraction of each node's min-marginal excess is handed over via
// give(i, k, h).  Returns the chain minimum (FP64).
template <class UN, class GIVE>
double chain_pass(int n, int D, const float *w, long wstride, const Rho &r, float slack, UN unary,
                  GIVE give, int32_t *labels, long lstride, std::vector<float> &Lbuf)
{
    Lbuf.assign((size_t)n * D, 0.0f);
    std::vector<float> L((size_t)D, 0.0f), v((size_t)D), R((size_t)D, 0.0f), m((size_t)D),
        A((size_t)D), tmp((size_t)D);
    // the chain minimum in FP64, summed in the GPU kernel's order: 32 partial
    // sums, partial l taking the node minima g_i with i = l mod 32 in ascending
    // i, then ((p0 + p1) + p2) + ... + p31
    double part[32] = {0.0};
    for (int i = 0; i < n; ++i) {
        std::memcpy(&Lbuf[(size_t)i * D], L.data(), sizeof(float) * D);
        for (int k = 0; k < D; ++k) v[k] = L[k] + unary(i, k);
        float g = vmin(v.data(), D);
        part[i & 31] += (double)g;
        if (i < n - 1) minconv(v.data(), g, w[(long)i * wstride], r, D, L.data());
    }
    double cmin = part[0];
    for (int l = 1; l < 32; ++l) cmin += part[l];
    for (int i = n - 1; i >= 0; --i) {
        for (int k = 0; k < D; ++k) {
            A[k] = unary(i, k);
            m[k] = (Lbuf[(size_t)i * D + k] + A[k]) + R[k];
        }
        float mu = vmin(m.data(), D);
        if (labels) {
            int best = 0;
            for (int k = 1; k < D; ++k)
                if (m[k] < m[best]) best = k;
            labels[(long)i * lstride] = best;
        }
        for (int k = 0; k < D; ++k) {
            float hk = slack * (m[k] - mu);
            A[k] = give(i, k, A[k], hk);
        }
        if (i > 0) {
            for (int k = 0; k < D; ++k) v[k] = A[k] + R[k];
            float g = vmin(v.data(), D);
            minconv(v.data(), g, w[(long)(i - 1) * wstride], r, D, tmp.data());
            R.swap(tmp);
        }
    }
    return cmin;
}

} // namespace

extern "C" {

int oracle_num_params(const oracle_cfg *cfg)
{
    return 2 * cfg->num_layers + (cfg->with_pairwise ? (cfg->topology == 2 ? 1 : 5) : 0);
}

int oracle_padding(const oracle_cfg *cfg)
{
    if (cfg->topology == 2) return growth_rate(cfg->num_layers) ? 0 : -1;
    int loss = 0;
    for (auto &L : feature_layers(cfg)) loss += L.kh - 1;
    if (loss % 2) return -1;
    return loss / 2;
}

int oracle_param_shape(const oracle_cfg *cfg, int i, int64_t shape[4], int *ndim)
{
    auto f = feature_layers(cfg);
    if (cfg->with_pairwise) {
        auto p = pairwise_layers(cfg);
        f.insert(f.end(), p.begin(), p.end());
    }
    for (auto &L : f) {
        if (L.wslot == i) {
            shape[0] = L.cout;
            shape[1] = L.cin;
            shape[2] = L.kh;
            shape[3] = L.kw;
            *ndim = 4;
            return 0;
        }
        if (L.bslot == i) {
            shape[0] = L.cout;
            *ndim = 1;
            return 0;
        }
    }
    return 1;
}

void oracle_xavier(const oracle_cfg *cfg, int i, uint64_t seed, float *out)
{
    int64_t s[4];
    int nd = 0;
    if (oracle_param_shape(cfg, i, s, &nd)) return;
    if (nd == 1) {
        for (int64_t j = 0; j < s[0]; ++j) out[j] = 0.0f;
        return;
    }
    cnncrf_xavier_fill(out, (int)s[0], (int)s[1], (int)s[2], (int)s[3], seed, i);
}

// stereo/stereo.cu:879-911 with cudaAddressModeMirror, point sampling at texel
// centres: symmetric reflection with the edge sample repeated.
static inline int mirror_idx(int i, int n)
{
    int m = i % (2 * n);
    if (m < 0) m += 2 * n;
    return m >= n ? 2 * n - 1 - m : m;
}

void oracle_pad_rgba(const float *in, int W, int H, int p, float *out)
{
    int Wp = W + 2 * p, Hp = H + 2 * p;
    for (int y = 0; y < Hp; ++y) {
        int sy = mirror_idx(y - p, H);
        for (int x = 0; x < Wp; ++x) {
            int sx = mirror_idx(x - p, W);
            std::memcpy(out + ((size_t)y * Wp + x) * 4, in + ((size_t)sy * W + sx) * 4, 16);
        }
    }
}

void oracle_normalize(const float *rgba, int Wp, int Hp, int ic, int precision, void *out)
{
    if (precision == 64) normalize_T<double>(rgba, Wp, Hp, ic, (double *)out);
    else normalize_T<float>(rgba, Wp, Hp, ic, (float *)out);
}

void oracle_conv(const void *in, int H, int W, int Cin, const float *w, const float *b, int Cout,
                 int kh, int kw, int act, int precision, void *out, int threads)
{
    set_threads(threads);
    if (precision == 64)
        conv_T<double>((const double *)in, H, W, Cin, w, b, Cout, kh, kw, act, (double *)out);
    else
        conv_T<float>((const float *)in, H, W, Cin, w, b, Cout, kh, kw, act, (float *)out);
}

void oracle_l2norm(void *f, long npx, int C, int precision)
{
    if (precision == 64) l2norm_T<double>((double *)f, npx, C);
    else l2norm_T<float>((float *)f, npx, C);
}

void oracle_correlation(const void *fl, const void *fr, int H, int W, int C, const float *list,
                        int D, int precision, void *out, int threads)
{
    set_threads(threads);
    if (precision == 64)
        correlation_T<double>((const double *)fl, (const double *)fr, H, W, C, list, D, 0,
                              (double *)out);
    else
        correlation_T<float>((const float *)fl, (const float *)fr, H, W, C, list, D, 0,
                             (float *)out);
}

void oracle_unary(void *vol, long npx, int D, int unary, int precision)
{
    if (precision == 64) unary_T<double>((double *)vol, npx, D, unary);
    else unary_T<float>((float *)vol, npx, D, unary);
}

// stereo/operators/stereocorrelation.cpp:83-85
int oracle_disparity_list(float min, float max, float step, float *list, int cap)
{
    int n = 0;
    for (float d = min; d <= max; d += step) {
        if (n < cap && list) list[n] = -d;
        ++n;
        if (n > 1 << 20) break;
    }
    return n;
}

// stereo/operators/stereocorrelation.cu:364-373 (element 1 is examined; a
// one-entry list examines element 0)
int oracle_disp_is_float(const float *list, int D)
{
    if (D <= 0) return 0;
    float v = D >= 2 ? list[1] : list[0];
    return std::fabs(v - std::round(v)) > 0.001f;
}

int oracle_predict(const oracle_cfg *cfg, const float *const *params, const float *left_pad,
                   const float *right_pad, int w, int h, const float *list, int D, void *vol,
                   void *pw)
{
    set_threads(cfg->threads);
    if (cfg->precision == 64)
        return predict_T<double>(cfg, params, left_pad, right_pad, w, h, list, D, 0, (double *)vol,
                                 (double *)pw);
    return predict_T<float>(cfg, params, left_pad, right_pad, w, h, list, D, 0, (float *)vol,
                            (float *)pw);
}

void oracle_crf(const float *cost, const float *wx, const float *wy, int W, int H, int D, float L1,
                float L2, int delta, int iters, int shape, float slack, int32_t *labels,
                double *lb, double *lb_iters, float *c1_out, int threads)
{
    set_threads(threads);
    Rho r = make_rho(L1, L2, delta, shape);
    size_t N = (size_t)W * H * D;
    std::vector<float> phi(N, 0.0f);
    std::vector<double> cH((size_t)H), cV((size_t)W);
    double lbv = 0.0;
    if (iters <= 0) {
        // degenerate: WTA (first minimum)
        for (long i = 0; i < (long)W * H; ++i) {
            int best = 0;
            for (int k = 1; k < D; ++k)
                if (cost[i * D + k] < cost[i * D + best]) best = k;
            if (labels) labels[i] = best;
        }
        if (lb) *lb = 0.0;
        return;
    }
    for (int it = 0; it < iters; ++it) {
        bool last = it == iters - 1;
#pragma omp parallel
        {
            std::vector<float> Lbuf;
#pragma omp for schedule(dynamic, 1)
            for (int y = 0; y < H; ++y) {
                const float *th = cost + (size_t)y * W * D;
                float *ph = phi.data() + (size_t)y * W * D;
                auto un = [&](int i, int k) { return th[(size_t)i * D + k] - ph[(size_t)i * D + k]; };
                auto give = [&](int i, int k, float a, float h) {
                    ph[(size_t)i * D + k] = ph[(size_t)i * D + k] + h;
                    return a - h;
                };
                cH[y] = chain_pass(W, D, wx + (size_t)y * W, 1, r, slack, un, give, nullptr, 0, Lbuf);
            }
#pragma omp for schedule(dynamic, 1)
            for (int x = 0; x < W; ++x) {
                float *ph = phi.data() + (size_t)x * D;
                long st = (long)W * D;
                auto un = [&](int i, int k) { return ph[(size_t)i * st + k]; };
                auto give = [&](int i, int k, float b, float h) {
                    float nb = b - h;
                    ph[(size_t)i * st + k] = nb;
                    return nb;
                };
                cV[x] = chain_pass(H, D, wy + x, W, r, slack, un, give,
                                   (last && labels) ? labels + x : nullptr, W, Lbuf);
            }
        }
        // each sum in the GPU's order (k_lb): 32 partial sums, partial l over the chains l, l + 32, ..
        // in ascending order, then the partials in order
        auto sum32 = [](const std::vector<double> &c) {
            double part[32] = {0.0};
            for (size_t i = 0; i < c.size(); ++i) part[i & 31] += c[i];
            double s = part[0];
            for (int l = 1; l < 32; ++l) s += part[l];
            return s;
        };
        lbv = sum32(cH) + sum32(cV);
        if (lb_iters) lb_iters[it] = lbv;
    }
    if (lb) *lb = lbv;
    if (c1_out)
        for (size_t i = 0; i < N; ++i) c1_out[i] = cost[i] - phi[i];
}

double oracle_energy(const float *cost, const float *wx, const float *wy, int W, int H, int D,
                     float L1, float L2, int delta, int shape, const int32_t *labels)
{
    Rho r = make_rho(L1, L2, delta, shape);
    auto rho = [&](int t) -> double {
        t = t < 0 ? -t : t;
        if (t == 0) return 0.0;
        if (t <= r.delta) return (double)r.rho[t];
        return (double)r.L2;
    };
    double e = 0.0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            long i = (long)y * W + x;
            e += (double)cost[i * D + labels[i]];
            if (x + 1 < W) e += (double)wx[i] * rho(labels[i] - labels[i + 1]);
            if (y + 1 < H) e += (double)wy[i] * rho(labels[i] - labels[i + W]);
        }
    return e;
}

double oracle_chain_bruteforce(const float *cost, const float *w, int n, int D, float L1, float L2,
                               int delta, int shape, int32_t *labels)
{
    Rho r = make_rho(L1, L2, delta, shape);
    auto rho = [&](int t) -> double {
        t = t < 0 ? -t : t;
        if (t == 0) return 0.0;
        if (t <= r.delta) return (double)r.rho[t];
        return (double)r.L2;
    };
    long total = 1;
    for (int i = 0; i < n; ++i) total *= D;
    double best = std::numeric_limits<double>::infinity();
    std::vector<int> x((size_t)n);
    for (long code = 0; code < total; ++code) {
        long c = code;
        for (int i = 0; i < n; ++i) {
            x[i] = (int)(c % D);
            c /= D;
        }
        double e = 0.0;
        for (int i = 0; i < n; ++i) {
            e += (double)cost[(size_t)i * D + x[i]];
            if (i + 1 < n) e += (double)w[i] * rho(x[i] - x[i + 1]);
        }
        if (e < best) {
            best = e;
            for (int i = 0; i < n; ++i) labels[i] = x[i];
        }
    }
    return best;
}

// stereo/stereo.cu:841-850
void oracle_remap(const int32_t *labels, long n, float dmin, float dstep, float *out)
{
    for (long i = 0; i < n; ++i) out[i] = ((float)labels[i] * dstep) + dmin;
}

// stereo/stereo.cu:348-370
void oracle_argmin(const float *vol, long npx, int D, float dmin, float dstep, float *out)
{
    for (long i = 0; i < npx; ++i) {
        float cm = FLT_MAX;
        int mi = 0;
        for (int z = 0; z < D; ++z)
            if (vol[i * D + z] < cm) {
                cm = vol[i * D + z];
                mi = z;
            }
        out[i] = dmin + (float)mi * dstep;
    }
}

// stereo/stereo.cu:830-839; the C4 texture is bound with point filtering and
// clamp addressing (stereo/stereo.cu:130-150,1138-1139): index floor(x+0.5-u).
void oracle_warp(const float *in, const float *u, int W, int H, float *out)
{
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float xf = ((float)x + 0.5f) - u[(size_t)y * W + x];
            int sx = (int)floorf(xf);
            sx = sx < 0 ? 0 : (sx > W - 1 ? W - 1 : sx);
            std::memcpy(out + ((size_t)y * W + x) * 4, in + ((size_t)y * W + sx) * 4, 16);
        }
}

// stereo/stereo.cu:419-442 with do_abs = false
void oracle_tv_fit(const float *vol3, int W, int H, float step, float lam, float *qf)
{
    float hh = step * 0.25f;
    for (long i = 0; i < (long)W * H; ++i) {
        float c0 = vol3[i * 3], c1 = vol3[i * 3 + 1], c2 = vol3[i * 3 + 2];
        float a = ((c0 - c2) / (hh * 2.0f)) * lam;
        float b = (((c0 + c2) - 2.0f * c1) / (hh * hh)) * lam;
        qf[i * 2] = a;
        qf[i * 2 + 1] = std::max(0.0f, b);
    }
}

static inline float clampf(float v, float lo, float hi) { return std::max(lo, std::min(v, hi)); }

// prox_p with alpha = 0 (stereo/stereo.cu:752-757)
static inline float prox_p0(float v, float beta, float sigma, float w)
{
    if (std::fabs(v) <= w * 0.0f) return v;
    float m = std::max(0.0f, fmaf(-sigma, beta, std::fabs(v)));
    float r = m * (v > 0.0f ? 1.0f : -1.0f);
    return clampf(r, -w, w);
}

// stereo/stereo.cu:701-729 (primal), 773-796 (dual), 1141-1143,1159-1166 (loop);
// the clamp-addressed texture reads become clamped indices.
void oracle_tv_iterate(float *u, float *u_, const float *u0, const float *qf, float *p, float *q,
                       const float *wx, const float *wy, int W, int H, float C, float eps,
                       float step, int iters)
{
    float L = (float)std::sqrt(8.0);
    float tau = 1.0f / L, sigma = 1.0f / L;
    float half = 0.5f * step;
    long N = (long)W * H;
    for (int it = 0; it < iters; ++it) {
        std::memcpy(u_, u, sizeof(float) * N);
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                long i = (long)y * W + x;
                long ixm = (long)y * W + (x > 0 ? x - 1 : 0);
                long iym = (long)(y > 0 ? y - 1 : 0) * W + x;
                float Px = p[2 * i] - q[2 * i], Py = p[2 * i + 1] - q[2 * i + 1];
                float X = p[2 * ixm] - q[2 * ixm];
                float Y = p[2 * iym + 1] - q[2 * iym + 1];
                float div = ((Px - X) + Py) - Y;
                float un = fmaf(tau, div, u[i]);
                float ax = qf[2 * i], by = qf[2 * i + 1];
                float uz = u0[i];
                float inner = fmaf(-by, uz, ax);
                float num = fmaf(-tau, inner, un);
                float den = fmaf(tau, by, 1.0f);
                un = clampf(num / den, uz - half, uz + half);
                u_[i] = 2.0f * un - u_[i];
                u[i] = un;
            }
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                long i = (long)y * W + x;
                float uc = u_[i];
                float dx = u_[(long)y * W + (x + 1 < W ? x + 1 : W - 1)] - uc;
                float dy = u_[(long)(y + 1 < H ? y + 1 : H - 1) * W + x] - uc;
                float pnx = fmaf(sigma, dx, p[2 * i]), pny = fmaf(sigma, dy, p[2 * i + 1]);
                float den = fmaf(sigma, eps, 1.0f);
                float wxx = wx[i], wyy = wy[i];
                p[2 * i] = clampf(pnx / den, -wxx, wxx);
                p[2 * i + 1] = clampf(pny / den, -wyy, wyy);
                float qnx = fmaf(sigma, dx, q[2 * i]), qny = fmaf(sigma, dy, q[2 * i + 1]);
                q[2 * i] = prox_p0(qnx, C, sigma, wxx);
                q[2 * i + 1] = prox_p0(qny, C, sigma, wyy);
            }
    }
}

// Stereo::computeVolume + computeSlackPropagation + fuseTHuberQuadFit
// (stereo/stereo.cpp:129-162,179-318,388-404; stereo/stereo.cu:1113-1170).
int oracle_run_pair(const oracle_cfg *cfg, const float *const *params, const float *left,
                    const float *right, int W, int H, float *disp, int32_t *labels, float *vol_out,
                    float *wx_out, float *wy_out, double *lb)
{
    set_threads(cfg->threads);
    int p = oracle_padding(cfg);
    if (p < 0 || (cfg->topology != 2 && p < 2 && cfg->with_pairwise)) return 1;
    int D = oracle_disparity_list(cfg->disp_min, cfg->disp_max, cfg->disp_step, nullptr, 0);
    std::vector<float> list((size_t)D);
    oracle_disparity_list(cfg->disp_min, cfg->disp_max, cfg->disp_step, list.data(), D);
    int w = W + 2 * p, h = H + 2 * p;
    std::vector<float> lp((size_t)w * h * 4), rp((size_t)w * h * 4);
    oracle_pad_rgba(left, W, H, p, lp.data());
    oracle_pad_rgba(right, W, H, p, rp.data());
    long N = (long)W * H;
    std::vector<float> vol((size_t)N * D), pw((size_t)2 * N, 0.0f);
    int rc;
    if (cfg->precision == 64) {
        std::vector<double> vd((size_t)N * D), pd((size_t)2 * N, 0.0);
        rc = predict_T<double>(cfg, params, lp.data(), rp.data(), w, h, list.data(), D, 0,
                               vd.data(), pd.data());
        for (size_t i = 0; i < vd.size(); ++i) vol[i] = (float)vd[i];
        for (size_t i = 0; i < pd.size(); ++i) pw[i] = (float)pd[i];
    } else {
        rc = predict_T<float>(cfg, params, lp.data(), rp.data(), w, h, list.data(), D, 0,
                              vol.data(), pw.data());
    }
    if (rc) return rc;
    std::vector<float> wx(pw.begin(), pw.begin() + N), wy(pw.begin() + N, pw.end());
    for (long i = 0; i < N; ++i) {
        wx[i] = wx[i] * cfg->lambda;
        wy[i] = wy[i] * cfg->lambda;
    }
    std::vector<int32_t> lab((size_t)N);
    double lbv = 0;
    oracle_crf(vol.data(), wx.data(), wy.data(), W, H, D, cfg->L1, cfg->L2, (int)cfg->delta,
               cfg->crf_iters, cfg->crf_shape, cfg->crf_slack, lab.data(), &lbv, nullptr, nullptr,
               cfg->threads);
    std::vector<float> u((size_t)N);
    oracle_remap(lab.data(), N, cfg->disp_min, cfg->disp_step, u.data());
    if (cfg->warps > 0 && cfg->with_pairwise) {
        float step = cfg->disp_step;
        float hq = (float)((double)step * 0.25);
        float mn = (float)(-(double)step * 0.25);
        int D3 = oracle_disparity_list(mn, hq, hq, nullptr, 0);
        std::vector<float> l3((size_t)D3);
        oracle_disparity_list(mn, hq, hq, l3.data(), D3);
        std::vector<float> u_((size_t)N), u0((size_t)N), qf((size_t)2 * N), pp((size_t)2 * N, 0.0f),
            qq((size_t)2 * N, 0.0f), warped((size_t)N * 4), wpad((size_t)w * h * 4),
            v3((size_t)N * D3), pw3((size_t)2 * N);
        float lam_c = 1.0f / cfg->lambda;
        for (int wi = 0; wi < cfg->warps; ++wi) {
            oracle_warp(right, u.data(), W, H, warped.data());
            oracle_pad_rgba(warped.data(), W, H, p, wpad.data());
            if (cfg->precision == 64) {
                std::vector<double> vd((size_t)N * D3), pd((size_t)2 * N);
                rc = predict_T<double>(cfg, params, lp.data(), wpad.data(), w, h, l3.data(), D3,
                                       cfg->refine_interp, vd.data(), pd.data());
                for (size_t i = 0; i < vd.size(); ++i) v3[i] = (float)vd[i];
                for (size_t i = 0; i < pd.size(); ++i) pw3[i] = (float)pd[i];
            } else {
                rc = predict_T<float>(cfg, params, lp.data(), wpad.data(), w, h, l3.data(), D3,
                                      cfg->refine_interp, v3.data(), pw3.data());
            }
            if (rc) return rc;
            // predict rewrote the pairwise buffer (wx, wy alias it) without lambda
            std::copy(pw3.begin(), pw3.begin() + N, wx.begin());
            std::copy(pw3.begin() + N, pw3.end(), wy.begin());
            if (D3 != 3) return 3;
            oracle_tv_fit(v3.data(), W, H, step, lam_c, qf.data());
            u0 = u;
            oracle_tv_iterate(u.data(), u_.data(), u0.data(), qf.data(), pp.data(), qq.data(),
                              wx.data(), wy.data(), W, H, cfg->C, cfg->huber_eps, step,
                              cfg->ref_iters);
        }
    }
    if (disp) std::copy(u.begin(), u.end(), disp);
    if (labels) std::copy(lab.begin(), lab.end(), labels);
    if (vol_out) std::copy(vol.begin(), vol.end(), vol_out);
    if (wx_out) std::copy(wx.begin(), wx.end(), wx_out);
    if (wy_out) std::copy(wy.begin(), wy.end(), wy_out);
    if (lb) *lb = lbv;
    return 0;
}

// ---------------------------------------------------------------- census, edges, QuadDirect, LR check
// (the reference reads these images through CUDA textures: clamp-addressed
// reads at integer positions, FP32 linear interpolation at fractional ones)

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

static inline float lerp_row(const float *r, int W, float u)
{
    const float t = u - 0.5f;
    const float f = std::floor(t);
    const int i = (int)f;
    const float a = t - f;
    const float v0 = r[clampi(i, 0, W - 1)];
    if (a == 0.0f) return v0;
    const float v1 = r[clampi(i + 1, 0, W - 1)];
    return v0 + a * (v1 - v0);
}

// rgb_to_gray_kernel (stereo/stereo.cu:853-863), weights in double, rounded once
void oracle_gray(const float *rgba, long n, float *gray)
{
    for (long i = 0; i < n; ++i) {
        const float *px = rgba + 4 * i;
        gray[i] = (float)(0.2989 * (double)px[0] + 0.5870 * (double)px[1] + 0.1140 * (double)px[2]);
    }
}

// cost_vol_census_kernel (stereo/stereo.cu:306-346)
void oracle_census(const float *g1, const float *g2, int W, int H, int fs, const float *list, int D, float lambda,
                   float *vol)
{
    const float norm = (float)(fs * fs * 4);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const float c1 = g1[(long)y * W + x];
            const float xx = (float)x + 0.5f;
            for (int z = 0; z < D; ++z) {
                const float d = list[z];
                const float c2 = lerp_row(g2 + (long)y * W, W, xx - d);
                float cnt = 0.0f;
                for (int dy = -fs; dy <= fs; ++dy) {
                    const int yy = clampi(y + dy, 0, H - 1);
                    const float *r1 = g1 + (long)yy * W, *r2 = g2 + (long)yy * W;
                    for (int dx = -fs; dx <= fs; ++dx) {
                        if (dx == 0 && dy == 0) continue;
                        const float i1 = r1[clampi(x + dx, 0, W - 1)];
                        const float i2 = lerp_row(r2, W, ((float)(x + dx) + 0.5f) - d);
                        if ((c1 > i1) != (c2 > i2)) cnt += 1.0f;
                    }
                }
                vol[((long)y * W + x) * D + z] = lambda * (cnt / norm);
            }
        }
}

// Gaussian weights exp(-i^2 / (2 sigma^2)) / sum, double, rounded once
void oracle_gauss_weights(float sigma, int R, float *w)
{
    double s = 0.0, v[64];
    for (int i = -R; i <= R; ++i) s += (v[i + R] = std::exp(-(double)(i * i) / (2.0 * sigma * sigma)));
    for (int i = 0; i <= 2 * R; ++i) w[i] = (float)(v[i] / s);
}

static inline float edge_weight(float diff, float alpha, float beta, float lambda)
{
    if (alpha > 0.0f)
        return std::max(cnncrf_mul(lambda, cnncrf_expf(cnncrf_mul(-alpha, cnncrf_powf(diff, beta)))), 1.0e-6f);
    return lambda * diff;
}

// calcEdgeImage (stereo/stereo.cu:1090-1095): Gaussian sigma 0.7 (radius 3,
// clamp-to-edge, horizontal then vertical), forward differences (the last
// column / row differs from itself: 0), edge weight of each difference
void oracle_edge_weights(const float *gray, int W, int H, float alpha, float beta, float lambda, float *wx,
                         float *wy)
{
    const int R = 3;
    float w[2 * R + 1];
    oracle_gauss_weights(0.7f, R, w);
    const long n = (long)W * H;
    std::vector<float> t1((size_t)n), t2((size_t)n);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float s = 0.0f;
            for (int i = -R; i <= R; ++i) s = fmaf(w[i + R], gray[(long)y * W + clampi(x + i, 0, W - 1)], s);
            t1[(long)y * W + x] = s;
        }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            float s = 0.0f;
            for (int i = -R; i <= R; ++i) s = fmaf(w[i + R], t1[(long)clampi(y + i, 0, H - 1) * W + x], s);
            t2[(long)y * W + x] = s;
        }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const long i = (long)y * W + x;
            const float c = t2[i];
            wx[i] = edge_weight(std::fabs(t2[(long)y * W + std::min(x + 1, W - 1)] - c), alpha, beta, lambda);
            wy[i] = edge_weight(std::fabs(t2[(long)std::min(y + 1, H - 1) * W + x] - c), alpha, beta, lambda);
        }
}

// do_fitting_kernel_volume + do_argmin_kernel_volume (stereo/stereo.cu:913-942)
void oracle_quadfit_direct(float *u, const float *c1, long npx, int D, float dmin, float dstep)
{
    for (long i = 0; i < npx; ++i) {
        const int z = (int)((u[i] - dmin) / dstep);
        if (z <= 0 || z >= D - 1) continue;
        const float *c = c1 + i * D;
        const float a = (c[z - 1] - c[z + 1]) / (dstep * 2.0f);
        const float b = std::max(1.0e-3f, ((c[z - 1] + c[z + 1]) - 2.0f * c[z]) / (dstep * dstep));
        u[i] = u[i] + a / b;
    }
}

// leftrightcheck_kernel (stereo/stereo.cu:803-817)
void oracle_lr_check(const float *left, const float *right, int W, int H, float th, float *out)
{
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const long i = (long)y * W + x;
            const float d = left[i];
            const float dr = -lerp_row(right + (long)y * W, W, ((float)x + 0.5f) - d);
            out[i] = std::fabs(d - dr) <= th ? d : -1.0f;
        }
}

} // extern "C"

// ================================================================ adjoints (training step), FP64
// The backward of oracle_predict for the one-minus-dot unary and integer
// disparity lists: given dL/dvol and dL/dpw, the gradient of every parameter
// in its npz layout.  The reference has no gradient code for the nets; the
// correlation adjoint follows the reference's backward kernels
// (stereo/operators/stereocorrelation.cu:210-350: dL/dfL and dL/dfR of the
// integer-disparity correlation, zero where x + s_k leaves the row).
namespace {

// Forward: out[oy][ox][co] = b[co] + sum_{ky,kx,ci} w[co][ci][kh-1-ky][kw-1-kx] in[oy+ky][ox+kx][ci].
// dz = dL/d(pre-activation output) [Ho][Wo][Cout].  Adds to dw (npz layout)
// and db (may be null); writes din [H][W][Cin] when non-null.
void conv_backward_d(const double *in, int H, int W, int Cin, const float *w, int Cout, int kh, int kw,
                     const double *dz, double *dw, double *db, double *din)
{
    const int Ho = H - kh + 1, Wo = W - kw + 1;
#pragma omp parallel for schedule(dynamic, 1)
    for (int co = 0; co < Cout; ++co) {
        for (int ci = 0; ci < Cin; ++ci)
            for (int ky = 0; ky < kh; ++ky)
                for (int kx = 0; kx < kw; ++kx) {
                    double acc = 0;
                    for (int oy = 0; oy < Ho; ++oy)
                        for (int ox = 0; ox < Wo; ++ox)
                            acc += dz[((size_t)oy * Wo + ox) * Cout + co] *
                                   in[((size_t)(oy + ky) * W + ox + kx) * Cin + ci];
                    dw[(((size_t)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)] += acc;
                }
        if (db) {
            double acc = 0;
            for (long i = 0; i < (long)Ho * Wo; ++i) acc += dz[(size_t)i * Cout + co];
            db[co] += acc;
        }
    }
    if (!din) return;
#pragma omp parallel for schedule(dynamic, 1)
    for (int iy = 0; iy < H; ++iy)
        for (int ix = 0; ix < W; ++ix) {
            double *d = din + ((size_t)iy * W + ix) * Cin;
            for (int ci = 0; ci < Cin; ++ci) d[ci] = 0;
            for (int ky = 0; ky < kh; ++ky) {
                const int oy = iy - ky;
                if (oy < 0 || oy >= Ho) continue;
                for (int kx = 0; kx < kw; ++kx) {
                    const int ox = ix - kx;
                    if (ox < 0 || ox >= Wo) continue;
                    const double *g = dz + ((size_t)oy * Wo + ox) * Cout;
                    for (int co = 0; co < Cout; ++co)
                        for (int ci = 0; ci < Cin; ++ci)
                            d[ci] += g[co] * (double)w[(((size_t)co * Cin + ci) * kh + (kh - 1 - ky)) * kw + (kw - 1 - kx)];
                }
            }
        }
}

// dz = dy * (1 - y^2), the tanh adjoint
void tanh_backward(const std::vector<double> &y, std::vector<double> &dy)
{
    for (size_t i = 0; i < y.size(); ++i) dy[i] *= 1.0 - y[i] * y[i];
}

size_t slot_size(const oracle_cfg *cfg, int i)
{
    int64_t s[4];
    int nd = 0;
    oracle_param_shape(cfg, i, s, &nd);
    size_t n = 1;
    for (int k = 0; k < nd; ++k) n *= (size_t)s[k];
    return n;
}

} // namespace

extern "C" {

/* grads[i]: slot i's gradient, slot_size doubles each, overwritten.
 * Returns 0, or 3 (unary is not one-minus-dot), 4 (fractional list), 1/2 (shape). */
int oracle_predict_backward(const oracle_cfg *cfg, const float *const *params, const float *lp, const float *rp,
                            int w, int h, const float *list, int D, const double *gvol, const double *gpw,
                            double *const *grads)
{
    if (cfg->unary != 1) return 3;
    if (oracle_disp_is_float(list, D)) return 4;
    if (cfg->topology == 2) return 5; // the concatenating net has no training path
    const int p = oracle_padding(cfg);
    if (p < 0) return 1;
    const int H = h - 2 * p, W = w - 2 * p, ic = cfg->in_channels, C = cfg->feat_channels;
    const int np = oracle_num_params(cfg);
    for (int i = 0; i < np; ++i) std::fill(grads[i], grads[i] + slot_size(cfg, i), 0.0);
    auto layers = feature_layers(cfg);
    const int L = (int)layers.size();
    // forward, keeping every layer's output
    std::vector<double> norm[2];
    std::vector<std::vector<double>> acts[2];
    std::vector<int> hs(L + 1), ws(L + 1);
    const float *img[2] = {lp, rp};
    for (int s = 0; s < 2; ++s) {
        norm[s].resize((size_t)w * h * ic);
        normalize_T<double>(img[s], w, h, ic, norm[s].data());
        acts[s].assign(L + 1, {});
        acts[s][0] = norm[s];
        int ch = h, cw = w;
        hs[0] = h, ws[0] = w;
        for (int l = 0; l < L; ++l) {
            const Layer &Ly = layers[l];
            const int oh = ch - Ly.kh + 1, ow = cw - Ly.kw + 1;
            acts[s][l + 1].assign((size_t)oh * ow * Ly.cout, 0.0);
            conv_T<double>(acts[s][l].data(), ch, cw, Ly.cin, params[Ly.wslot], params[Ly.bslot], Ly.cout, Ly.kh,
                           Ly.kw, 1, acts[s][l + 1].data());
            ch = oh, cw = ow;
            hs[l + 1] = ch, ws[l + 1] = cw;
        }
        if (ch != H || cw != W) return 2;
    }
    // L2 normalisation (kept: f and the norms)
    std::vector<double> f[2], nrm[2];
    for (int s = 0; s < 2; ++s) {
        f[s] = acts[s][L];
        nrm[s].assign((size_t)H * W, 0.0);
        for (long i = 0; i < (long)H * W; ++i) {
            double *q = f[s].data() + i * C;
            double ss = 0;
            for (int c = 0; c < C; ++c) ss = std::fma(q[c], q[c], ss);
            const double n = std::sqrt(ss);
            nrm[s][i] = n;
            for (int c = 0; c < C; ++c) q[c] = n > 0 ? q[c] / n : 0.0;
        }
    }
    // correlation adjoint: vol = 1 - C, so dC = -gvol
    std::vector<double> df[2];
    df[0].assign((size_t)H * W * C, 0.0);
    df[1].assign((size_t)H * W * C, 0.0);
#pragma omp parallel for
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            for (int k = 0; k < D; ++k) {
                const int xs = x + (int)list[k];
                if (xs < 0 || xs > W - 1) continue;
                const double g = -gvol[((size_t)y * W + x) * D + k];
                const double *a = f[0].data() + ((size_t)y * W + x) * C;
                const double *b = f[1].data() + ((size_t)y * W + xs) * C;
                double *da = df[0].data() + ((size_t)y * W + x) * C;
                double *dbb = df[1].data() + ((size_t)y * W + xs) * C;
                for (int c = 0; c < C; ++c) {
                    da[c] += g * b[c];
                    dbb[c] += g * a[c];
                }
            }
    // through the normalisation, the tanh layers and the convolutions of both images
    for (int s = 0; s < 2; ++s) {
        std::vector<double> dy((size_t)H * W * C);
        for (long i = 0; i < (long)H * W; ++i) {
            const double *q = f[s].data() + i * C, *g = df[s].data() + i * C;
            double dot = 0;
            for (int c = 0; c < C; ++c) dot += q[c] * g[c];
            const double n = nrm[s][i];
            for (int c = 0; c < C; ++c) dy[(size_t)i * C + c] = n > 0 ? (g[c] - q[c] * dot) / n : 0.0;
        }
        for (int l = L - 1; l >= 0; --l) {
            const Layer &Ly = layers[l];
            tanh_backward(acts[s][l + 1], dy);
            std::vector<double> din;
            if (l > 0) din.assign((size_t)hs[l] * ws[l] * Ly.cin, 0.0);
            conv_backward_d(acts[s][l].data(), hs[l], ws[l], Ly.cin, params[Ly.wslot], Ly.cout, Ly.kh, Ly.kw,
                            dy.data(), grads[Ly.wslot], grads[Ly.bslot], l > 0 ? din.data() : nullptr);
            dy.swap(din);
        }
    }
    if (cfg->with_pairwise && gpw) {
        const int cr = p - 2, pc = ic == 1 ? 1 : 3, ph = H + 4, pww = W + 4;
        std::vector<double> pin((size_t)ph * pww * pc);
        for (int y = 0; y < ph; ++y)
            for (int x = 0; x < pww; ++x)
                for (int c = 0; c < pc; ++c)
                    pin[((size_t)y * pww + x) * pc + c] = norm[0][((size_t)(y + cr) * w + x + cr) * ic + c];
        auto pl = pairwise_layers(cfg);
        const Layer &A = pl[0], &B = pl[1], &Hd = pl[2];
        std::vector<double> y1((size_t)(H + 2) * (W + 2) * A.cout), y2((size_t)H * W * B.cout), hh((size_t)H * W * 2);
        conv_T<double>(pin.data(), ph, pww, A.cin, params[A.wslot], params[A.bslot], A.cout, 3, 3, 1, y1.data());
        conv_T<double>(y1.data(), H + 2, W + 2, B.cin, params[B.wslot], params[B.bslot], B.cout, 3, 3, 1, y2.data());
        conv_T<double>(y2.data(), H, W, Hd.cin, params[Hd.wslot], nullptr, 2, 1, 1, 0, hh.data());
        std::vector<double> gh((size_t)H * W * 2);
        for (long i = 0; i < (long)H * W; ++i)
            for (int o = 0; o < 2; ++o) {
                const double v = hh[(size_t)i * 2 + o];
                const double sg = v > 0 ? 1.0 : (v < 0 ? -1.0 : 0.0); // d|v|/dv
                gh[(size_t)i * 2 + o] = gpw[(size_t)o * H * W + i] * sg;
            }
        std::vector<double> dy2((size_t)H * W * B.cout), dy1((size_t)(H + 2) * (W + 2) * A.cout);
        conv_backward_d(y2.data(), H, W, Hd.cin, params[Hd.wslot], 2, 1, 1, gh.data(), grads[Hd.wslot], nullptr,
                        dy2.data());
        tanh_backward(y2, dy2);
        conv_backward_d(y1.data(), H + 2, W + 2, B.cin, params[B.wslot], B.cout, 3, 3, dy2.data(), grads[B.wslot],
                        grads[B.bslot], dy1.data());
        tanh_backward(y1, dy1);
        conv_backward_d(pin.data(), ph, pww, A.cin, params[A.wslot], A.cout, 3, 3, dy1.data(), grads[A.wslot],
                        grads[A.bslot], nullptr);
    }
    return 0;
}

} // extern "C"
