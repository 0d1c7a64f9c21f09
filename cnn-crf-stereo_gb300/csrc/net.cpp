// net.cpp -- StereoNet / ColorStereoNet: layer bookkeeping, parameters,
// disparities and predict() over the CUDA kernels (C ABI cnncrf_net_*).
//
// Reference: stereo/stereonet.cpp (initNet 65-182, setAllParams 184-227,
// setDisparities 229-248, performPrediction 250-421) and
// stereo/colorstereonet.cpp:38-133 (predict / predictXY).
#include "net.h"

#include <cmath>
#include <cstring>

#include "../../include/cnncrf_xavier.h"
#include "kernels.h"
#include "npz.h"

using namespace cnncrf;

namespace {

constexpr int NPAD = 128; // output-channel padding of the FP32 weight layout

// float -> bfloat16, round to nearest even
uint16_t f2bf(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;
    u += 0x7fffu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

int pad_to(int c, int m) { return (c + m - 1) / m * m; }

// UMMA N for a layer width: 64, 112 or 128
int umma_n(int cout) { return cout <= 64 ? 64 : (cout <= 112 ? 112 : 128); }

void build_layers(cnncrf_net *n)
{
    const cnncrf_net_desc &d = n->d;
    int F = d.feat_channels;
    n->feat.clear();
    n->pw.clear();
    if (d.topology == CNNCRF_TOPO_CONCAT) {
        // stereo/concatstereonet.cpp:72-127: 3x3 convs to the growth rate g, each
        // fed the previous layer's g channels, every layer tanh; the pairwise
        // weights one 3x3 conv of the concatenated features to 2 channels, no bias,
        // |tanh| (non-negative, as the CRF needs)
        const int g = n->growth;
        n->feat.push_back({d.in_channels, g, 3, 3, 1, 0, 1});
        for (int l = 1; l < d.num_layers; ++l) n->feat.push_back({g, g, 3, 3, 1, 2 * l, 2 * l + 1});
        if (d.with_pairwise) n->pw.push_back({F, 2, 3, 3, 3, 2 * d.num_layers, -1});
        const int nparams = 2 * d.num_layers + (d.with_pairwise ? 1 : 0);
        n->host.assign(nparams, {});
        n->have.assign(nparams, 0);
        return;
    }
    // stereo/stereonet.cpp:69-133: 3x3 first, 2x2 after (REF), every layer tanh
    n->feat.push_back({d.in_channels, F, 3, 3, 1, 0, 1});
    int k = d.topology == CNNCRF_TOPO_REF ? 2 : 3;
    for (int l = 1; l < d.num_layers; ++l) n->feat.push_back({F, F, k, k, 1, 2 * l, 2 * l + 1});
    if (d.with_pairwise) { // stereo/stereonet.cpp:159-167
        int base = 2 * d.num_layers, pc = d.in_channels == 1 ? 1 : 3, P = d.pw_channels;
        n->pw.push_back({pc, P, 3, 3, 1, base, base + 1});
        n->pw.push_back({P, P, 3, 3, 1, base + 2, base + 3});
        n->pw.push_back({P, 2, 1, 1, 2, base + 4, -1});
    }
    int nparams = 2 * d.num_layers + (d.with_pairwise ? 5 : 0);
    n->host.assign(nparams, {});
    n->have.assign(nparams, 0);
}

cnncrf_net::Layer *layer_of_slot(cnncrf_net *n, int slot, bool *is_bias)
{
    for (auto *v : {&n->feat, &n->pw})
        for (auto &L : *v) {
            if (L.wslot == slot) {
                *is_bias = false;
                return &L;
            }
            if (L.bslot == slot) {
                *is_bias = true;
                return &L;
            }
        }
    return nullptr;
}

} // namespace

int cnncrf_net::expected_shape(int i, int64_t s[4], int *nd) const
{
    bool b;
    auto *L = layer_of_slot(const_cast<cnncrf_net *>(this), i, &b);
    if (!L) return fail(CNNCRF_EINVAL, "parameter index %d outside 0..%d", i, num_params() - 1);
    if (b) {
        s[0] = L->cout;
        *nd = 1;
    } else {
        s[0] = L->cout, s[1] = L->cin, s[2] = L->kh, s[3] = L->kw;
        *nd = 4;
    }
    return CNNCRF_OK;
}

// Upload the device copies of the layer owning `slot`.
int cnncrf_net::upload(int slot)
{
    bool isb;
    Layer *L = layer_of_slot(this, slot, &isb);
    if (!L) return fail(CNNCRF_EINVAL, "no layer for slot %d", slot);
    const std::vector<float> &src = host[slot];
    if (isb) {
        std::vector<float> b(NPAD, 0.0f);
        for (int co = 0; co < L->cout; ++co) b[co] = src[co];
        CNNCRF_TRY(L->bias.reserve(NPAD * sizeof(float)));
        CNNCRF_CUDA(cudaMemcpy(L->bias.get(), b.data(), NPAD * sizeof(float), cudaMemcpyHostToDevice));
        return CNNCRF_OK;
    }
    if (L->kh == 1 && L->kw == 1 && L->cout == 2) { // pairwise head: [2][Cin]
        std::vector<float> w(2 * L->cin);
        for (int co = 0; co < 2; ++co)
            for (int ci = 0; ci < L->cin; ++ci) w[co * L->cin + ci] = src[co * L->cin + ci];
        CNNCRF_TRY(L->wt.reserve(w.size() * sizeof(float)));
        CNNCRF_CUDA(cudaMemcpy(L->wt.get(), w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice));
        if (d.precision == CNNCRF_BF16) { // [2][np] for the fused head of the tensor-core conv
            int np = umma_n(L->cin);
            std::vector<float> h((size_t)2 * np, 0.0f);
            for (int co = 0; co < 2; ++co)
                for (int ci = 0; ci < L->cin; ++ci) h[(size_t)co * np + ci] = src[co * L->cin + ci];
            CNNCRF_TRY(head16.reserve(h.size() * sizeof(float)));
            CNNCRF_CUDA(cudaMemcpy(head16.get(), h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
        }
        return CNNCRF_OK;
    }
    // CUDNN_CONVOLUTION flips the kernel: wt[(ky*kw+kx)*Cin+ci][co] = w[co][ci][kh-1-ky][kw-1-kx]
    int K = L->kh * L->kw * L->cin;
    std::vector<float> wt((size_t)K * NPAD, 0.0f);
    for (int co = 0; co < L->cout; ++co)
        for (int ci = 0; ci < L->cin; ++ci)
            for (int ky = 0; ky < L->kh; ++ky)
                for (int kx = 0; kx < L->kw; ++kx) {
                    int k = (ky * L->kw + kx) * L->cin + ci;
                    wt[(size_t)k * NPAD + co] =
                        src[(((size_t)co * L->cin + ci) * L->kh + (L->kh - 1 - ky)) * L->kw + (L->kw - 1 - kx)];
                }
    CNNCRF_TRY(L->wt.reserve(wt.size() * sizeof(float)));
    CNNCRF_CUDA(cudaMemcpy(L->wt.get(), wt.data(), wt.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (d.precision == CNNCRF_BF16 && L->cin >= 16) {
        // tensor-core layout: [np][tap][cp] BF16, K-major per output channel
        int np = umma_n(L->cout), cp = pad_to(L->cin, 64), taps = L->kh * L->kw;
        std::vector<uint16_t> w16((size_t)np * taps * cp, 0);
        for (int co = 0; co < L->cout; ++co)
            for (int ky = 0; ky < L->kh; ++ky)
                for (int kx = 0; kx < L->kw; ++kx)
                    for (int ci = 0; ci < L->cin; ++ci)
                        w16[((size_t)co * taps + ky * L->kw + kx) * cp + ci] = f2bf(
                            src[(((size_t)co * L->cin + ci) * L->kh + (L->kh - 1 - ky)) * L->kw + (L->kw - 1 - kx)]);
        CNNCRF_TRY(L->wt16.reserve(w16.size() * 2));
        CNNCRF_CUDA(cudaMemcpy(L->wt16.get(), w16.data(), w16.size() * 2, cudaMemcpyHostToDevice));
    }
    return CNNCRF_OK;
}

// StereoCorrelation::setDisparities (stereo/operators/stereocorrelation.cpp:71-144)
int cnncrf_net::set_disparities(float mn, float mx, float step, float *d_out)
{
    if (!(step > 0.0f)) return fail(CNNCRF_EINVAL, "setDisparities: step must be > 0");
    std::vector<float> l;
    for (float dd = mn; dd <= mx; dd += step) {
        l.push_back(-dd);
        if (l.size() > 4096) return fail(CNNCRF_EINVAL, "setDisparities: more than 4096 disparities");
    }
    if (l.empty()) return fail(CNNCRF_EINVAL, "setDisparities: empty range [%g, %g]", mn, mx);
    list = l;
    D = (int)l.size();
    float v = D >= 2 ? l[1] : l[0]; // stereo/operators/stereocorrelation.cu:364-373
    interp = std::fabs(v - std::round(v)) > 0.001f;
    bool ip = interp || force_interp;
    int_list = true;
    for (float s : l) int_list = int_list && s == std::floor(s);
    omin = 1 << 30, omax = -(1 << 30);
    for (float s : l) {
        int a, b;
        if (ip) {
            a = (int)std::floor(s) - 1;
            b = (int)std::floor(s) + 2;
        } else {
            a = b = (int)s;
        }
        omin = std::min(omin, a);
        omax = std::max(omax, b);
    }
    CNNCRF_TRY(d_list.reserve(sizeof(float) * D));
    CNNCRF_CUDA(cudaMemcpy(d_list.get(), l.data(), sizeof(float) * D, cudaMemcpyHostToDevice));
    if (d_out) {
        vol = d_out;
    } else {
        CNNCRF_TRY(vol_own.reserve(sizeof(float) * (size_t)H * W * D * n));
        vol = vol_own.as<float>();
    }
    return CNNCRF_OK;
}

int cnncrf_net::pairwise_fp32()
{
    // crop by pad-2 of the normalised left image (stereo/colorstereonet.cpp:69-73)
    int cr = pad - 2, ic = d.in_channels, P = d.pw_channels;
    const float *in = norm[0].as<float>() + ((size_t)cr * w + cr) * ic;
    k::ConvArgs a1{in, H + 4, W + 4, pw[0].cin, (long)ic, (long)w * ic, pw[0].wt.as<float>(),
                   pw[0].bias.as<float>(), pw[0].cout, 3, 3, 1, pwa.as<float>()};
    a1.n_img = n, a1.in_img = (long)h * w * ic, a1.out_img = (long)(H + 2) * (W + 2) * P;
    CNNCRF_TRY(k::conv_simt(a1, st));
    k::ConvArgs a2{pwa.as<float>(), H + 2, W + 2, pw[1].cin, (long)pw[1].cin, (long)(W + 2) * pw[1].cin,
                   pw[1].wt.as<float>(), pw[1].bias.as<float>(), pw[1].cout, 3, 3, 1, pwb.as<float>()};
    a2.n_img = n, a2.in_img = (long)(H + 2) * (W + 2) * P, a2.out_img = (long)H * W * P;
    CNNCRF_TRY(k::conv_simt(a2, st));
    return k::conv_head2(pwb.as<float>(), H * W, pw[2].cin, pw[2].wt.as<float>(), pwout, st, n);
}

int cnncrf_net::predict_fp32(const float *left, const float *right, bool reuse_left_features)
{
    const float *img[2] = {left, right};
    int ic = d.in_channels;
    const bool reuse = reuse_left_features && left_ok;
    left_ok = false;
    for (int s = 0; s < 2; ++s) {
        if (s == 0 && reuse) continue; // feats[0] and norm[0] still hold this input's features
        CNNCRF_TRY(k::normalize(img[s], w, h, ic, norm[s].as<float>(), scratch.get(), st, n));
        const float *cur = norm[s].as<float>();
        int ch = h, cw = w, cc = ic;
        for (size_t l = 0; l < feat.size(); ++l) {
            Layer &L = feat[l];
            float *out = act[s][l & 1].as<float>();
            k::ConvArgs a{cur, ch, cw, cc, (long)cc, (long)cw * cc, L.wt.as<float>(), L.bias.as<float>(),
                          L.cout, L.kh, L.kw, L.act, out};
            int oh = ch - (L.kh - 1), ow = cw - (L.kw - 1);
            a.n_img = n, a.in_img = (long)ch * cw * cc, a.out_img = (long)oh * ow * L.cout;
            CNNCRF_TRY(k::conv_simt(a, st));
            ch = oh, cw = ow, cc = L.cout;
            cur = out;
        }
        feats[s] = const_cast<float *>(cur);
        if (d.unary == CNNCRF_UNARY_ONE_MINUS_DOT)
            CNNCRF_TRY(k::l2norm(feats[s], (long)H * W * n, d.feat_channels, st));
    }
    CNNCRF_TRY(k::correlation(feats[0], feats[1], H, W, d.feat_channels, d_list.as<float>(), D, omin, omax,
                              interp || force_interp, d.unary, vol, st, n, (long)H * W * d.feat_channels));
    if (d.with_pairwise) CNNCRF_TRY(pairwise_fp32());
    left_ok = true;
    return CNNCRF_OK;
}

// ConcatStereoNet (FP32): every layer a 3x3 conv with zero padding 1 to the
// growth rate g.  Layer l writes channels [l g, (l+1) g) of one zero-bordered
// tensor cz [n][h+2][w+2][g L] and reads layer l-1's channels of it, so the
// border supplies the padding and the concatenation needs no copy.  The
// correlation reads the features cropped to [n][H][W][g L]; the pairwise conv
// reads the bordered left features (before any L2 normalisation).
int cnncrf_net::predict_concat(const float *left, const float *right)
{
    const float *img[2] = {left, right};
    const int ic = d.in_channels, C = d.feat_channels, g = growth;
    const long bw = w + 2, bh = h + 2;
    const long x_img = bh * bw * ic, z_img = bh * bw * C;
    for (int s = 0; s < 2; ++s) {
        CNNCRF_TRY(k::normalize(img[s], w, h, ic, norm[s].as<float>(), scratch.get(), st, n));
        float *x = cx[s].as<float>(), *z = cz[s].as<float>();
        for (int i = 0; i < n; ++i)
            CNNCRF_CUDA(cudaMemcpy2DAsync(x + i * x_img + (bw + 1) * ic, sizeof(float) * bw * ic,
                                          norm[s].as<float>() + (long)i * h * w * ic, sizeof(float) * w * ic,
                                          sizeof(float) * w * ic, h, cudaMemcpyDeviceToDevice, st));
        for (size_t l = 0; l < feat.size(); ++l) {
            Layer &L = feat[l];
            const bool first = l == 0;
            k::ConvArgs a{first ? x : z + (l - 1) * g, (int)bh, (int)bw, L.cin, first ? (long)ic : (long)C,
                          bw * (first ? ic : C), L.wt.as<float>(), L.bias.as<float>(), L.cout, 3, 3, L.act,
                          z + (bw + 1) * C + (long)l * g};
            a.n_img = n, a.in_img = first ? x_img : z_img, a.out_img = z_img;
            a.out_pix = C, a.out_row = bw * C, a.out_ch = 1;
            CNNCRF_TRY(k::conv_simt(a, st));
        }
        for (int i = 0; i < n; ++i)
            CNNCRF_CUDA(cudaMemcpy2DAsync(cf[s].as<float>() + (long)i * H * W * C, sizeof(float) * W * C,
                                          z + i * z_img + (bw + 1) * C, sizeof(float) * bw * C, sizeof(float) * W * C,
                                          H, cudaMemcpyDeviceToDevice, st));
        feats[s] = cf[s].as<float>();
    }
    if (d.with_pairwise) {
        Layer &P = pw[0];
        k::ConvArgs a{cz[0].as<float>(), (int)bh, (int)bw, C, (long)C, bw * C, P.wt.as<float>(), nullptr, 2, 3, 3,
                      P.act, pwout};
        a.n_img = n, a.in_img = z_img, a.out_img = 2L * H * W;
        a.out_pix = 1, a.out_row = W, a.out_ch = (long)H * W; // planar [2][H][W]
        CNNCRF_TRY(k::conv_simt(a, st));
    }
    if (d.unary == CNNCRF_UNARY_ONE_MINUS_DOT)
        for (int s = 0; s < 2; ++s) CNNCRF_TRY(k::l2norm(feats[s], (long)H * W * n, C, st));
    return k::correlation(feats[0], feats[1], H, W, C, d_list.as<float>(), D, omin, omax, interp || force_interp,
                          d.unary, vol, st, n, (long)H * W * C);
}

int cnncrf_net::predict(const float *left, const float *right)
{
    if (!inited) return fail(CNNCRF_ESTATE, "predict before initNet");
    for (size_t i = 0; i < have.size(); ++i)
        if (!have[i]) return fail(CNNCRF_ESTATE, "parameter arr_%zu not set", i);
    if (!left || !right) return fail(CNNCRF_EINVAL, "predict: null image");
    volq_valid = false;
    const bool reuse = reuse_left;
    reuse_left = false;
    if (d.topology == CNNCRF_TOPO_CONCAT || d.precision == CNNCRF_BF16) {
        left_ok = false;
        return d.topology == CNNCRF_TOPO_CONCAT ? predict_concat(left, right) : predict_bf16(left, right);
    }
    return predict_fp32(left, right, reuse);
}

int cnncrf::concat_growth(int layers)
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

int cnncrf::net_padding(const cnncrf_net_desc &d)
{
    if (d.topology == CNNCRF_TOPO_CONCAT) return 0;
    const int loss = 2 + (d.num_layers - 1) * (d.topology == CNNCRF_TOPO_REF ? 1 : 2);
    return loss / 2;
}

// ---------------------------------------------------------------- C ABI

extern "C" {

int cnncrf_net_create(cnncrf_net_t *out, const cnncrf_net_desc *desc, int n, int h, int w)
{
    clear_error();
    if (!out || !desc) return fail(CNNCRF_EINVAL, "net_create: null argument");
    *out = nullptr;
    const cnncrf_net_desc &d = *desc;
    if (n < 1 || n > 256) return fail(CNNCRF_EINVAL, "net_create: batch n = %d outside 1..256", n);
    const bool concat = d.topology == CNNCRF_TOPO_CONCAT;
    if (d.topology != CNNCRF_TOPO_REF && d.topology != CNNCRF_TOPO_ALL3X3 && !concat)
        return fail(CNNCRF_EINVAL, "net_create: topology %d", d.topology);
    const int growth = concat ? concat_growth(d.num_layers) : 0;
    if (concat && growth == 0) // stereo/concatstereonet.cpp:52-55
        return fail(CNNCRF_EINVAL, "ConcatStereoNet must have one of the following numbers of layers: 3, 5, 7, 10, "
                                   "15, 20, 25, 33, 50, 100 (got %d)", d.num_layers);
    if (!concat && (d.num_layers < 1 || d.num_layers > 16))
        return fail(CNNCRF_EINVAL, "net_create: num_layers %d", d.num_layers);
    if (d.in_channels != 1 && d.in_channels != 3 && d.in_channels != 5)
        return fail(CNNCRF_EINVAL, "net_create: in_channels must be 1, 3 or 5");
    if (concat && d.feat_channels != 0 && d.feat_channels != growth * d.num_layers)
        return fail(CNNCRF_EINVAL, "net_create: the concatenating net's features are %d x %d = %d channels, not %d",
                    d.num_layers, growth, growth * d.num_layers, d.feat_channels);
    if (!concat && (d.feat_channels < 1 || d.feat_channels > 128))
        return fail(CNNCRF_EINVAL, "net_create: feat_channels %d outside 1..128", d.feat_channels);
    if (d.with_pairwise && (d.pw_channels < 1 || d.pw_channels > 128))
        return fail(CNNCRF_EINVAL, "net_create: pw_channels %d outside 1..128", d.pw_channels);
    if (d.unary != CNNCRF_UNARY_NEG_SOFTMAX && d.unary != CNNCRF_UNARY_ONE_MINUS_DOT)
        return fail(CNNCRF_EINVAL, "net_create: unary %d", d.unary);
    if (d.precision != CNNCRF_FP32 && d.precision != CNNCRF_BF16)
        return fail(CNNCRF_EINVAL, "net_create: precision %d", d.precision);
    if (concat && d.precision != CNNCRF_FP32)
        return fail(CNNCRF_EUNSUPPORTED, "net_create: the concatenating net runs in FP32 only");
    auto *net = new cnncrf_net;
    net->d = d;
    if (concat) {
        net->growth = growth;
        net->d.feat_channels = growth * d.num_layers;
        build_layers(net);
        net->pad = 0; // stereo/stereo.cpp:214-216
        net->n = n, net->h = h, net->w = w, net->H = h, net->W = w;
        if (h < 1 || w < 1) {
            delete net;
            return fail(CNNCRF_ESHAPE, "net_create: empty %dx%d input", w, h);
        }
        *out = net;
        return CNNCRF_OK;
    }
    build_layers(net);
    int loss = 0;
    for (auto &L : net->feat) loss += L.kh - 1;
    if (loss % 2) {
        delete net;
        return fail(CNNCRF_EINVAL, "net_create: receptive-field loss %d is odd", loss);
    }
    net->pad = loss / 2;
    if (d.with_pairwise && net->pad < 2) {
        delete net;
        return fail(CNNCRF_EINVAL, "net_create: pairwise net needs padding >= 2");
    }
    net->n = n, net->h = h, net->w = w;
    net->H = h - 2 * net->pad, net->W = w - 2 * net->pad;
    if (net->H < 1 || net->W < 1) {
        delete net;
        return fail(CNNCRF_ESHAPE, "net_create: padded input %dx%d smaller than the receptive field", w, h);
    }
    *out = net;
    return CNNCRF_OK;
}

int cnncrf_net_destroy(cnncrf_net_t net)
{
    delete net;
    return CNNCRF_OK;
}

int cnncrf_net_set_stream(cnncrf_net_t net, cnncrf_stream_t stream)
{
    if (!net) return fail(CNNCRF_EINVAL, "null net");
    net->st = (cudaStream_t)stream;
    return CNNCRF_OK;
}

int cnncrf_net_init(cnncrf_net_t net, float min_disp, float max_disp, float step, int rect_corr,
                    float *d_unary_out, float *d_pairwise_out)
{
    clear_error();
    if (!net) return fail(CNNCRF_EINVAL, "null net");
    if (rect_corr != 0) return fail(CNNCRF_EUNSUPPORTED, "rect_corr != 0 is not built");
    int ic = net->d.in_channels, h = net->h, w = net->w, H = net->H, W = net->W, nb = net->n;
    size_t np = (size_t)h * w * nb;
    for (int s = 0; s < 2; ++s) CNNCRF_TRY(net->norm[s].reserve(np * ic * sizeof(float)));
    size_t amax = 0;
    if (net->d.topology != CNNCRF_TOPO_CONCAT) { // valid convs: each layer shrinks the maps
        int ch = h, cw = w;
        for (auto &L : net->feat) {
            ch -= L.kh - 1, cw -= L.kw - 1;
            amax = std::max(amax, (size_t)ch * cw * L.cout);
        }
    }
    const bool fp32 = net->d.precision == CNNCRF_FP32;
    const bool concat = net->d.topology == CNNCRF_TOPO_CONCAT;
    for (int s = 0; s < 2; ++s)
        for (int b = 0; b < 2; ++b)
            if (fp32 && !concat) CNNCRF_TRY(net->act[s][b].reserve(amax * nb * sizeof(float)));
    if (concat) { // the borders stay zero: predict writes only the interiors
        const size_t bpx = (size_t)(h + 2) * (w + 2) * nb, C = net->d.feat_channels;
        for (int s = 0; s < 2; ++s) {
            CNNCRF_TRY(net->cx[s].reserve(bpx * ic * sizeof(float)));
            CNNCRF_TRY(net->cz[s].reserve(bpx * C * sizeof(float)));
            CNNCRF_TRY(net->cf[s].reserve((size_t)H * W * nb * C * sizeof(float)));
            CNNCRF_CUDA(cudaMemsetAsync(net->cx[s].get(), 0, bpx * ic * sizeof(float), net->st));
            CNNCRF_CUDA(cudaMemsetAsync(net->cz[s].get(), 0, bpx * C * sizeof(float), net->st));
        }
    }
    CNNCRF_TRY(net->scratch.reserve(k::normalize_scratch_bytes(h, nb)));
    if (net->d.with_pairwise) {
        int P = net->d.pw_channels;
        if (fp32 && !concat) {
            CNNCRF_TRY(net->pwa.reserve((size_t)(H + 2) * (W + 2) * P * nb * sizeof(float)));
            CNNCRF_TRY(net->pwb.reserve((size_t)H * W * P * nb * sizeof(float)));
        }
        if (d_pairwise_out) {
            net->pwout = d_pairwise_out;
        } else {
            CNNCRF_TRY(net->pw_own.reserve((size_t)2 * H * W * nb * sizeof(float)));
            net->pwout = net->pw_own.as<float>();
        }
    }
    if (net->d.precision == CNNCRF_BF16) CNNCRF_TRY(net->alloc_bf16());
    CNNCRF_TRY(net->set_disparities(min_disp, max_disp, step, d_unary_out));
    net->inited = true;
    return CNNCRF_OK;
}

int cnncrf_net_set_param(cnncrf_net_t net, int index, const float *h_data, const int64_t *shape, int ndim)
{
    clear_error();
    if (!net || !h_data || !shape) return fail(CNNCRF_EINVAL, "set_param: null argument");
    int64_t s[4];
    int nd;
    CNNCRF_TRY(net->expected_shape(index, s, &nd));
    // a 1-D bias may arrive as (C,) ; a filter must match (co, ci, kh, kw)
    bool ok = ndim == nd;
    for (int i = 0; ok && i < nd; ++i) ok = shape[i] == s[i];
    if (!ok) {
        std::string got, want;
        for (int i = 0; i < ndim; ++i) got += std::to_string(shape[i]) + " ";
        for (int i = 0; i < nd; ++i) want += std::to_string(s[i]) + " ";
        return fail(CNNCRF_ESHAPE, "arr_%d: loaded shape (%s) but the layer needs (%s)", index, got.c_str(),
                    want.c_str());
    }
    size_t cnt = 1;
    for (int i = 0; i < nd; ++i) cnt *= (size_t)s[i];
    net->host[index].assign(h_data, h_data + cnt);
    net->have[index] = 1;
    return net->upload(index);
}

int cnncrf_net_set_all_params(cnncrf_net_t net, const char *npz_path)
{
    clear_error();
    if (!net || !npz_path) return fail(CNNCRF_EINVAL, "set_all_params: null argument");
    for (int i = 0; i < net->num_params(); ++i) {
        NpyArray a;
        CNNCRF_TRY(npz_load(npz_path, "arr_" + std::to_string(i), &a));
        CNNCRF_TRY(cnncrf_net_set_param(net, i, a.data.data(), a.shape.data(), (int)a.shape.size()));
    }
    return CNNCRF_OK;
}

int cnncrf_net_num_params(cnncrf_net_t net, int *count)
{
    if (!net || !count) return fail(CNNCRF_EINVAL, "null argument");
    *count = net->num_params();
    return CNNCRF_OK;
}

int cnncrf_net_param_shape(cnncrf_net_t net, int index, int64_t shape[4], int *ndim)
{
    if (!net || !shape || !ndim) return fail(CNNCRF_EINVAL, "null argument");
    return net->expected_shape(index, shape, ndim);
}

int cnncrf_net_init_xavier(cnncrf_net_t net, uint64_t seed)
{
    clear_error();
    if (!net) return fail(CNNCRF_EINVAL, "null net");
    for (int i = 0; i < net->num_params(); ++i) {
        int64_t s[4];
        int nd;
        CNNCRF_TRY(net->expected_shape(i, s, &nd));
        std::vector<float> v;
        if (nd == 1) {
            v.assign((size_t)s[0], 0.0f);
        } else {
            v.resize((size_t)(s[0] * s[1] * s[2] * s[3]));
            cnncrf_xavier_fill(v.data(), (int)s[0], (int)s[1], (int)s[2], (int)s[3], seed, i);
        }
        CNNCRF_TRY(cnncrf_net_set_param(net, i, v.data(), s, nd));
    }
    return CNNCRF_OK;
}

int cnncrf_net_set_disparities(cnncrf_net_t net, float min_disp, float max_disp, float step, float *d_out)
{
    clear_error();
    if (!net) return fail(CNNCRF_EINVAL, "null net");
    return net->set_disparities(min_disp, max_disp, step, d_out);
}

int cnncrf_net_num_disparities(cnncrf_net_t net, int *num)
{
    if (!net || !num) return fail(CNNCRF_EINVAL, "null argument");
    *num = net->D;
    return CNNCRF_OK;
}

int cnncrf_net_predict(cnncrf_net_t net, const float *d_left_rgba, const float *d_right_rgba, float **d_volume)
{
    CNNCRF_RANGE("net_predict");
    clear_error();
    if (!net) return fail(CNNCRF_EINVAL, "null net");
    CNNCRF_TRY(net->predict(d_left_rgba, d_right_rgba));
    if (d_volume) *d_volume = net->vol;
    return CNNCRF_OK;
}

int cnncrf_net_pairwise(cnncrf_net_t net, float **d_pairwise)
{
    if (!net || !d_pairwise) return fail(CNNCRF_EINVAL, "null argument");
    if (!net->d.with_pairwise) return fail(CNNCRF_ESTATE, "net has no pairwise CNN");
    *d_pairwise = net->pwout;
    return CNNCRF_OK;
}

int cnncrf_net_features(cnncrf_net_t net, int side, float *d_out)
{
    if (!net || !d_out || side < 0 || side > 1) return fail(CNNCRF_EINVAL, "features: bad argument");
    if (net->d.precision == CNNCRF_BF16) {
        if (!net->feat16) return fail(CNNCRF_ESTATE, "features: no prediction yet");
        size_t npx = (size_t)net->H * net->W;
        const uint16_t *f = (const uint16_t *)net->feat16 + (size_t)side * net->n * npx * net->cp_feat;
        return k::bf16_to_f32(f, net->cp_feat, net->d.feat_channels, (long)npx, d_out, net->st);
    }
    if (!net->feats[side]) return fail(CNNCRF_ESTATE, "features: no prediction yet");
    CNNCRF_CUDA(cudaMemcpyAsync(d_out, net->feats[side], sizeof(float) * (size_t)net->H * net->W * net->d.feat_channels,
                                cudaMemcpyDeviceToDevice, net->st));
    return CNNCRF_OK;
}

int cnncrf_net_padding(cnncrf_net_t net, int *pad)
{
    if (!net || !pad) return fail(CNNCRF_EINVAL, "null argument");
    *pad = net->pad;
    return CNNCRF_OK;
}

} // extern "C"
