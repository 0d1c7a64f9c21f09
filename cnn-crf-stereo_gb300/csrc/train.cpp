// train.cpp -- the training step (cnncrf_train_*): forward through both
// nets and the correlation keeping every layer's activations, the structured
// hinge loss on the CRF's loss-augmented labelling, the backward through the
// hand-written adjoints (k_train.cu) into every parameter, SGD with momentum
// on FP32 master weights.
//
// No counterpart in the reference, which ships inference only (its weights
// were trained elsewhere).  The forward is StereoNet::performPrediction
// (stereo/stereonet.cpp:250-421) on the FP32 kernels of the inference path,
// so the volume and the pairwise output equal the inference net's bit for
// bit; padding and normalisation are those of ColorStereoNet::predict
// (stereo/colorstereonet.cpp:38-77).  One-minus-dot unary, integer disparity
// list, RGB input.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cnncrf.h"
#include "../../include/cnncrf_xavier.h"
#include "common.h"
#include "kernels.h"
#include "npz.h"

using namespace cnncrf;

namespace {

struct TLayer {
    int cin, cout, kh, kw, act, wslot, bslot;
    int hin, win;        // input extent
    DevBuf wt, wd, b128; // conv_simt layout, input-gradient layout, padded bias
    DevBuf w16;          // the BF16 mode's tensor-core layout
    DevBuf w16d;         // its input-gradient layout (tensor-core input gradients)
    bool tcw = false;    // the weight gradient on the tensor cores
    bool dprev = false;  // the backward pass computes this layer's input gradient
    int hout() const { return hin - kh + 1; }
    int wout() const { return win - kw + 1; }
};

size_t al64(size_t x) { return (x + 63) & ~(size_t)63; }

} // namespace

struct cnncrf_train {
    cnncrf_train_desc d{};
    int n = 0, H = 0, W = 0, p = 0, h = 0, w = 0, D = 0;
    const int ic = 3;
    bool bf16 = false;
    int cp_feat = 0, np_feat = 0, cp_pw = 0, np_pw = 0;
    cudaStream_t st = nullptr;
    std::vector<TLayer> feat, pw; // pw: conv 3x3, conv 3x3, 1x1 head
    std::vector<size_t> off, cnt; // slot offset / count in the flat parameter buffers
    size_t total = 0;
    DevBuf theta, grad, vel;
    std::vector<float> list;
    int omin = 0, omax = 0;
    DevBuf dlist;
    // forward state.  The feature net runs both sides as one batch of 2n images (left crops, then right):
    // every feature buffer holds both sides, and its side s is the half at s * n images.
    // Feature-layer outputs: checkpoints in their own buffers, the rest in a shared pool.
    DevBuf padded, norm, scratch;
    DevBuf norm16; // BF16 copy of norm at channel stride 64 (the first layers' tensor-core weight gradients)
    bool tc_corr = false; // the correlation adjoint on the tensor cores
    std::vector<char> keep;
    std::vector<DevBuf> act, pool;
    DevBuf fbuf, vol, y1, y2, pwout; // fbuf: both sides' normalised features
    bool forwarded = false, hinged = false;
    // backward and hinge scratch
    DevBuf gvol, gpw, df, dy, dyb, padb, part, partb, gh; // df: both sides' feature gradients
    DevBuf aug, wts, labels, crfws, contrib, rows, err, tcerr;
    size_t crfws_bytes = 0;
    DevBuf wgs; // the tensor-core weight gradient's planar copies and partial sums
    size_t wgs_bytes = 0;
    // the BF16 padded output gradient that the tensor-core weight and input gradients read; two, since a
    // fused input gradient writes the layer below's copy while reading its own
    DevBuf dpad[2];
    int dcur = 0;
    // the per-channel sums of the ready dz (the fused input gradient's epilogue): bsplits rows of scratch
    DevBuf bpart;
    int bsplits = 0;
    bool bias_ready = false;

    int build();
    int refresh();
    int forward(const float *l, const float *r);
    int hinge(const int32_t *gt, double *loss, int32_t *yh_out);
    int backward(const float *gv, const float *gp);
    int run_layer(int l);
    int layer_back(TLayer &L, int nimg, const void *in, bool in_bf16, long in_pix, long in_row, long in_img,
                   const void *y, int ys, float *dz, float *dprev, bool &ready, const TLayer *below);
    int nf() const { return 2 * n; } // images of the feature net: both sides
    float *norm_s(int s) { return norm.as<float>() + (size_t)s * n * h * w * ic; }
    float *padded_s(int s) { return padded.as<float>() + (size_t)s * n * h * w * 4; }
    float *df_s(int s) { return df.as<float>() + (size_t)s * n * H * W * d.feat_channels; }
    float *param(int slot) { return theta.as<float>() + off[slot]; }
    float *gradp(int slot) { return grad.as<float>() + off[slot]; }
    size_t es() const { return bf16 ? 2 : 4; }
    int fstride() const { return bf16 ? cp_feat : d.feat_channels; } // channel stride of feature activations
    int pstride() const { return bf16 ? cp_pw : d.pw_channels; }
    void *actp(int l) // layer l's output, both sides
    {
        if (keep[l]) return act[l].get();
        int c = l;
        while (c > 0 && !keep[c - 1]) --c; // first layer of l's segment
        return pool[l - c].get();
    }
    void *fside(int s) { return (char *)fbuf.get() + (size_t)s * n * H * W * fstride() * es(); }
};

namespace {
int pad_to(int c, int m) { return (c + m - 1) / m * m; }
int umma_n(int cout) { return cout <= 64 ? 64 : (cout <= 112 ? 112 : 128); }
} // namespace

int cnncrf_train::build()
{
    const int L = d.num_layers, F = d.feat_channels, P = d.pw_channels;
    const int k = d.topology == CNNCRF_TOPO_REF ? 2 : 3;
    bf16 = d.precision == CNNCRF_BF16;
    if (bf16 && (L < 2 || F < 16 || P < 16))
        return fail(CNNCRF_EUNSUPPORTED, "train: the BF16 mode needs >= 2 layers and >= 16 channels per net");
    cp_feat = bf16 ? pad_to(F, 64) : F, np_feat = umma_n(F);
    cp_pw = bf16 ? pad_to(P, 64) : P, np_pw = umma_n(P);
    feat.clear();
    pw.clear();
    feat.push_back({ic, F, 3, 3, 1, 0, 1, 0, 0}); // stereo/stereonet.cpp:69-79
    for (int l = 1; l < L; ++l) feat.push_back({F, F, k, k, 1, 2 * l, 2 * l + 1, 0, 0});
    for (int l = 1; l < L; ++l) feat[l].dprev = true;
    int loss = 0;
    for (auto &Ly : feat) loss += Ly.kh - 1;
    if (loss % 2) return fail(CNNCRF_EINVAL, "train: receptive-field loss %d is odd", loss);
    p = loss / 2;
    if (p < 2) return fail(CNNCRF_EINVAL, "train: the pairwise net needs padding >= 2");
    h = H + 2 * p, w = W + 2 * p;
    int ch = h, cw = w;
    for (auto &Ly : feat) {
        Ly.hin = ch, Ly.win = cw;
        ch -= Ly.kh - 1, cw -= Ly.kw - 1;
    }
    const int base = 2 * L; // stereo/stereonet.cpp:159-167
    pw.push_back({3, P, 3, 3, 1, base, base + 1, H + 4, W + 4});
    pw.push_back({P, P, 3, 3, 1, base + 2, base + 3, H + 2, W + 2});
    pw.push_back({P, 2, 1, 1, 2, base + 4, -1, H, W});
    pw[1].dprev = true;
    const int np = 2 * L + 5;
    off.assign(np, 0);
    cnt.assign(np, 0);
    for (auto *v : {&feat, &pw})
        for (auto &Ly : *v) {
            cnt[Ly.wslot] = (size_t)Ly.cout * Ly.cin * Ly.kh * Ly.kw;
            if (Ly.bslot >= 0) cnt[Ly.bslot] = Ly.cout;
        }
    total = 0;
    for (int i = 0; i < np; ++i) {
        off[i] = total;
        total += al64(cnt[i]);
    }
    for (auto *b : {&theta, &grad, &vel}) {
        CNNCRF_TRY(b->reserve(total * sizeof(float)));
        CNNCRF_CUDA(cudaMemset(b->get(), 0, total * sizeof(float)));
    }
    for (auto *v : {&feat, &pw})
        for (auto &Ly : *v)
            if (Ly.act == 1) {
                CNNCRF_TRY(Ly.wt.reserve(sizeof(float) * (size_t)Ly.kh * Ly.kw * Ly.cin * 128));
                CNNCRF_TRY(Ly.wd.reserve(sizeof(float) * (size_t)Ly.kh * Ly.kw * Ly.cout * 128));
                CNNCRF_TRY(Ly.b128.reserve(sizeof(float) * 128));
                CNNCRF_CUDA(cudaMemset(Ly.b128.get(), 0, sizeof(float) * 128));
                if (bf16 && Ly.cin >= 16) { // the tensor-core layers
                    const int npd = v == &feat ? np_feat : np_pw, cpi = v == &feat ? cp_feat : cp_pw;
                    CNNCRF_TRY(Ly.w16.reserve(2 * (size_t)npd * Ly.kh * Ly.kw * cpi));
                    if (d.tc_dgrad && Ly.cout <= 128 && Ly.kw <= 3)
                        CNNCRF_TRY(Ly.w16d.reserve(2 * (size_t)umma_n(Ly.cin) * Ly.kh * Ly.kw * pad_to(Ly.cout, 64)));
                }
            }
    // the stored list -d (stereo/operators/stereocorrelation.cpp:83-85); integers only
    list.clear();
    for (float dd = d.disp_min; dd <= d.disp_max; dd += d.disp_step) {
        list.push_back(-dd);
        if (list.size() > 256) return fail(CNNCRF_EINVAL, "train: more than 256 disparities");
    }
    if (list.empty()) return fail(CNNCRF_EINVAL, "train: empty disparity range");
    D = (int)list.size();
    omin = 1 << 30, omax = -(1 << 30);
    for (float s : list) {
        if (s != std::floor(s)) return fail(CNNCRF_EUNSUPPORTED, "train: fractional disparity %g", -s);
        omin = std::min(omin, (int)s), omax = std::max(omax, (int)s);
    }
    CNNCRF_TRY(dlist.reserve(sizeof(float) * D));
    CNNCRF_CUDA(cudaMemcpy(dlist.get(), list.data(), sizeof(float) * D, cudaMemcpyHostToDevice));
    // checkpoints: every r-th feature layer's output and the last one; the rest is recomputed in backward
    const int r = d.checkpoint_every;
    keep.assign(L, 1);
    if (r > 0)
        for (int l = 0; l < L; ++l) keep[l] = (l + 1) % r == 0 || l == L - 1;
    int run = 0, poolsz = 0;
    for (int l = 0; l < L; ++l) {
        run = keep[l] ? 0 : run + 1;
        poolsz = std::max(poolsz, run);
    }
    // activations (zeroed: the BF16 mode's padding channels must read as zero)
    const size_t N = (size_t)n * H * W;
    size_t amax = (size_t)n * h * w * 4, lmax = 0;
    for (auto &Ly : feat) lmax = std::max(lmax, (size_t)nf() * Ly.hout() * Ly.wout() * fstride() * es());
    auto zalloc = [&](DevBuf &b, size_t bytes) -> int {
        CNNCRF_TRY(b.reserve(bytes));
        CNNCRF_CUDA(cudaMemset(b.get(), 0, bytes));
        return CNNCRF_OK;
    };
    CNNCRF_TRY(padded.reserve(sizeof(float) * nf() * h * w * 4));
    CNNCRF_TRY(norm.reserve(sizeof(float) * nf() * h * w * ic));
    act.clear();
    act.resize(feat.size());
    for (size_t l = 0; l < feat.size(); ++l) {
        const size_t e = (size_t)nf() * feat[l].hout() * feat[l].wout() * F;
        amax = std::max(amax, e);
        if (keep[l]) CNNCRF_TRY(zalloc(act[l], (size_t)nf() * feat[l].hout() * feat[l].wout() * fstride() * es()));
    }
    CNNCRF_TRY(df.reserve(sizeof(float) * 2 * N * F));
    pool.clear();
    pool.resize(poolsz);
    for (auto &b : pool) CNNCRF_TRY(zalloc(b, lmax));
    CNNCRF_TRY(zalloc(fbuf, 2 * N * fstride() * es()));
    CNNCRF_TRY(scratch.reserve(k::normalize_scratch_bytes(h, n)));
    CNNCRF_TRY(vol.reserve(sizeof(float) * N * D));
    CNNCRF_TRY(zalloc(y1, (size_t)n * (H + 2) * (W + 2) * pstride() * es()));
    CNNCRF_TRY(zalloc(y2, N * pstride() * es()));
    CNNCRF_TRY(pwout.reserve(sizeof(float) * N * 2));
    amax = std::max(amax, (size_t)n * (H + 4) * (W + 4) * P);
    // backward: dy / dyb hold any layer's output or input gradient, padb a padded output gradient
    CNNCRF_TRY(dy.reserve(sizeof(float) * amax));
    CNNCRF_TRY(dyb.reserve(sizeof(float) * amax));
    CNNCRF_TRY(padb.reserve(sizeof(float) * (size_t)nf() * (h + 4) * (w + 4) * std::max(F, P)));
    CNNCRF_TRY(gvol.reserve(sizeof(float) * N * D));
    CNNCRF_TRY(gpw.reserve(sizeof(float) * N * 2));
    CNNCRF_TRY(gh.reserve(sizeof(float) * N * 2));
    long Pmax = 0;
    size_t part_floats = 0;
    for (auto *v : {&feat, &pw})
        for (auto &Ly : *v) {
            const long P = (long)(v == &feat ? nf() : n) * Ly.hout() * Ly.wout();
            const int K = Ly.kh * Ly.kw * Ly.cin;
            Pmax = std::max(Pmax, P);
            part_floats = std::max(part_floats, (size_t)k::train_wgrad_splits_k(P, K) * Ly.cout * K);
        }
    // the BF16 mode's tensor-core weight gradients: scratch for the largest layer
    if (bf16 && d.tc_wgrad)
        for (auto *v : {&feat, &pw})
            for (auto &Ly : *v)
                if (Ly.act == 1 && k::wgrad_tc_supported(Ly.cout, Ly.cin, Ly.kh, Ly.kw)) {
                    const long steps = (long)(v == &feat ? nf() : n) * Ly.hout() * ((Ly.wout() + 63) / 64);
                    wgs_bytes = std::max(wgs_bytes, k::wgrad_tc_scratch_bytes(Ly.cout, Ly.cin, Ly.kh, Ly.kw,
                                                                              k::wgrad_tc_splits(Ly.kh, steps)));
                    Ly.tcw = true;
                }
    if (wgs_bytes) CNNCRF_TRY(wgs.reserve(wgs_bytes));
    tc_corr = bf16 && d.tc_dgrad && k::corr_bwd_tc_supported(F, cp_feat, D, omin, omax);
    if (feat[0].tcw || pw[0].tcw)
        CNNCRF_TRY(zalloc(norm16, 2 * (size_t)nf() * h * w * 64));
    size_t dpad_bytes = 0;
    for (auto *v : {&feat, &pw})
        for (auto &Ly : *v)
            if (Ly.w16d.get() || Ly.tcw)
                dpad_bytes = std::max(dpad_bytes, 2 * (size_t)(v == &feat ? nf() : n) * (Ly.hout() + 2 * (Ly.kh - 1)) *
                                                      (Ly.wout() + 2 * (Ly.kw - 1)) * pad_to(Ly.cout, 64));
    if (dpad_bytes) {
        for (auto &b : dpad) CNNCRF_TRY(zalloc(b, dpad_bytes));
        int dev = 0, sms = 0;
        CNNCRF_CUDA(cudaGetDevice(&dev));
        CNNCRF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        CNNCRF_TRY(bpart.reserve(sizeof(float) * 8 * (size_t)sms * 128)); // conv_tc: 8 rows per CTA
    }
    const int ns = k::train_wgrad_splits(Pmax); // the most bias splits any layer uses
    CNNCRF_TRY(part.reserve(sizeof(float) * part_floats));
    CNNCRF_TRY(partb.reserve(sizeof(float) * (size_t)ns * 128));
    // hinge
    CNNCRF_TRY(aug.reserve(sizeof(float) * N * D));
    CNNCRF_TRY(wts.reserve(sizeof(float) * N * 2));
    CNNCRF_TRY(labels.reserve(sizeof(int32_t) * N));
    crfws_bytes = k::crf_workspace_bytes(W, H, D, n);
    CNNCRF_TRY(crfws.reserve(crfws_bytes));
    CNNCRF_TRY(contrib.reserve(sizeof(double) * N));
    CNNCRF_TRY(rows.reserve(sizeof(double) * n * H));
    CNNCRF_TRY(zalloc(err, sizeof(int)));
    CNNCRF_TRY(zalloc(tcerr, sizeof(int)));
    return CNNCRF_OK;
}

// the kernel layouts of every weight from the master copy
int cnncrf_train::refresh()
{
    for (auto *v : {&feat, &pw})
        for (auto &Ly : *v)
            if (Ly.act == 1) {
                CNNCRF_TRY(k::train_weight_layouts(param(Ly.wslot), param(Ly.bslot), Ly.cout, Ly.cin, Ly.kh, Ly.kw,
                                                   Ly.wt.as<float>(), Ly.wd.as<float>(), Ly.b128.as<float>(), st));
                if (Ly.w16.get())
                    CNNCRF_TRY(k::train_w16(param(Ly.wslot), Ly.cout, Ly.cin, Ly.kh, Ly.kw,
                                            v == &feat ? np_feat : np_pw, v == &feat ? cp_feat : cp_pw, Ly.w16.get(),
                                            st));
                if (Ly.w16d.get())
                    CNNCRF_TRY(k::train_w16_dgrad(param(Ly.wslot), Ly.cout, Ly.cin, Ly.kh, Ly.kw, umma_n(Ly.cin),
                                                  pad_to(Ly.cout, 64), Ly.w16d.get(), st));
            }
    return CNNCRF_OK;
}

// feature layer l of both sides into actp(l)
int cnncrf_train::run_layer(int l)
{
    TLayer &Ly = feat[l];
    void *out = actp(l);
    if (l == 0 || !bf16) {
        const float *in = l == 0 ? norm.as<float>() : (const float *)actp(l - 1);
        const int cs = l == 0 ? ic : d.feat_channels;
        k::ConvArgs a{in, Ly.hin, Ly.win, Ly.cin, (long)cs, (long)Ly.win * cs, Ly.wt.as<float>(), Ly.b128.as<float>(),
                      Ly.cout, Ly.kh, Ly.kw, 1, bf16 ? nullptr : (float *)out};
        a.n_img = nf(), a.in_img = (long)Ly.hin * Ly.win * cs, a.out_img = (long)Ly.hout() * Ly.wout() * fstride();
        if (!bf16) return k::conv_simt(a, st);
        a.out16 = out, a.out_cs = cp_feat; // BF16 NHWC output padded to cp_feat
        return k::conv_first_tc_supported(a) ? k::conv_first_tc(a, tcerr.as<int>(), st) : k::conv_simt(a, st);
    }
    k::TcConvArgs t{};
    t.in = actp(l - 1);
    t.n_img = nf(), t.Hin = Ly.hin, t.Win = Ly.win, t.cp_in = cp_feat, t.cin = Ly.cin;
    t.wt = Ly.w16.get();
    t.np = np_feat, t.cout = Ly.cout, t.kh = Ly.kh, t.kw = Ly.kw;
    t.bias = Ly.b128.as<float>();
    t.head = nullptr;
    t.mode = 0; // tanh -> BF16: the pre-normalisation features stay for the backward
    t.out = out;
    t.cp_out = cp_feat;
    if (l == (int)feat.size() - 1) { // the last layer also writes the L2-normalised features
        t.mode = 1, t.out = fbuf.get(); // both sides, in the order the correlation reads them
        t.out16 = out, t.o16_cs = cp_feat;
    }
    t.err = tcerr.as<int>();
    return k::conv_tc(t, st);
}

int cnncrf_train::forward(const float *l, const float *r)
{
    const float *img[2] = {l, r};
    const int F = d.feat_channels, L = (int)feat.size();
    for (int s = 0; s < 2; ++s) {
        CNNCRF_TRY(k::pad_rgba(img[s], W, H, p, padded_s(s), st, n));
        CNNCRF_TRY(k::normalize(padded_s(s), w, h, ic, norm_s(s), scratch.get(), st, n));
    }
    if (norm16.get()) CNNCRF_TRY(k::train_to_bf16_c64(norm.as<float>(), (long)nf() * h * w, ic, norm16.get(), st));
    for (int li = 0; li < L; ++li) CNNCRF_TRY(run_layer(li)); // both sides at once
    if (!bf16) { // (the BF16 last layer's epilogue wrote the normalised features)
        const size_t fb = sizeof(float) * (size_t)nf() * H * W * F;
        CNNCRF_CUDA(cudaMemcpyAsync(fbuf.get(), actp(L - 1), fb, cudaMemcpyDeviceToDevice, st));
        CNNCRF_TRY(k::l2norm(fbuf.as<float>(), (long)nf() * H * W, F, st));
    }
    if (!bf16)
        CNNCRF_TRY(k::correlation((const float *)fside(0), (const float *)fside(1), H, W, F, dlist.as<float>(), D, omin,
                                  omax, false, CNNCRF_UNARY_ONE_MINUS_DOT, vol.as<float>(), st, n, (long)H * W * F));
    else if (k::corr_tc_supported(F, cp_feat, list.data(), D, CNNCRF_UNARY_ONE_MINUS_DOT))
        CNNCRF_TRY(k::correlation_tc(fbuf.get(), n, H, W, F, cp_feat, dlist.as<float>(), list.data(), D,
                                     CNNCRF_UNARY_ONE_MINUS_DOT, vol.as<float>(), tcerr.as<int>(), st));
    else
        CNNCRF_TRY(k::correlation_bf16(fside(0), fside(1), H, W, F, cp_feat, dlist.as<float>(), D, omin, omax, false,
                                       CNNCRF_UNARY_ONE_MINUS_DOT, vol.as<float>(), st, n, (long)H * W * cp_feat));
    // pairwise net on the left image's normalisation cropped by p - 2 (stereo/colorstereonet.cpp:69-73)
    const int cr = p - 2, P = d.pw_channels;
    const float *in = norm_s(0) + ((size_t)cr * w + cr) * ic;
    k::ConvArgs a1{in, H + 4, W + 4, 3, (long)ic, (long)w * ic, pw[0].wt.as<float>(), pw[0].b128.as<float>(), P, 3, 3,
                   1, bf16 ? nullptr : y1.as<float>()};
    a1.n_img = n, a1.in_img = (long)h * w * ic, a1.out_img = (long)(H + 2) * (W + 2) * pstride();
    if (!bf16) {
        CNNCRF_TRY(k::conv_simt(a1, st));
        k::ConvArgs a2{y1.as<float>(), H + 2, W + 2, P, (long)P, (long)(W + 2) * P, pw[1].wt.as<float>(),
                       pw[1].b128.as<float>(), P, 3, 3, 1, y2.as<float>()};
        a2.n_img = n, a2.in_img = (long)(H + 2) * (W + 2) * P, a2.out_img = (long)H * W * P;
        CNNCRF_TRY(k::conv_simt(a2, st));
        CNNCRF_TRY(k::conv_head2(y2.as<float>(), H * W, P, param(pw[2].wslot), pwout.as<float>(), st, n));
    } else {
        a1.out16 = y1.get(), a1.out_cs = cp_pw;
        CNNCRF_TRY(k::conv_first_tc_supported(a1) ? k::conv_first_tc(a1, tcerr.as<int>(), st) : k::conv_simt(a1, st));
        k::TcConvArgs t{};
        t.in = y1.get();
        t.n_img = n, t.Hin = H + 2, t.Win = W + 2, t.cp_in = cp_pw, t.cin = P;
        t.wt = pw[1].w16.get();
        t.np = np_pw, t.cout = P, t.kh = 3, t.kw = 3;
        t.bias = pw[1].b128.as<float>();
        t.err = tcerr.as<int>();
        if (np_pw == P) { // the head and |.| in the epilogue ([2][P] weights = [2][NP]), y2 beside it
            t.mode = 2, t.head = param(pw[2].wslot), t.out = pwout.get(), t.cp_out = 0;
            t.out16 = y2.get(), t.o16_cs = cp_pw;
            CNNCRF_TRY(k::conv_tc(t, st));
        } else {
            t.mode = 0, t.out = y2.get(), t.cp_out = cp_pw;
            CNNCRF_TRY(k::conv_tc(t, st));
            CNNCRF_TRY(k::train_head2_bf16(y2.get(), n, H * W, P, cp_pw, param(pw[2].wslot), pwout.as<float>(), st));
        }
    }
    forwarded = true;
    hinged = false;
    return CNNCRF_OK;
}

int cnncrf_train::hinge(const int32_t *gt, double *loss, int32_t *yh_out)
{
    if (!forwarded) return fail(CNNCRF_ESTATE, "train: hinge before forward");
    const long N = (long)n * H * W;
    CNNCRF_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), st));
    CNNCRF_TRY(k::train_augment(vol.as<float>(), gt, N, D, aug.as<float>(), err.as<int>(), st));
    CNNCRF_CUDA(cudaMemcpyAsync(wts.get(), pwout.get(), sizeof(float) * N * 2, cudaMemcpyDeviceToDevice, st));
    CNNCRF_TRY(k::scale(wts.as<float>(), N * 2, d.lambda, st)); // stereo/stereo.cpp:136-137
    k::CrfParams cp;
    cp.L1 = d.L1, cp.L2 = d.L2, cp.delta = d.delta, cp.shape = d.crf_shape, cp.slack = d.crf_slack;
    CNNCRF_TRY(k::crf_solve_batch(aug.as<float>(), wts.as<float>(), W, H, D, n, cp, d.crf_iters, labels.as<int32_t>(),
                                  crfws.get(), crfws_bytes, st, false)); // labels and bounds only
    float rho[9];
    rho[0] = 0.0f;
    for (int t = 1; t <= 8; ++t) rho[t] = d.crf_shape == 0 ? fminf(d.L1, d.L2) : fminf(d.L1 * (float)t, d.L2);
    CNNCRF_CUDA(cudaMemsetAsync(gvol.get(), 0, sizeof(float) * N * D, st));
    // mean loss: every pair's loss per pixel, the subgradient of their mean over the batch
    const float gscale = d.mean_loss ? (float)(1.0 / (double)N) : 1.0f;
    CNNCRF_TRY(k::train_hinge(vol.as<float>(), wts.as<float>(), gt, labels.as<int32_t>(), n, W, H, D, d.lambda, rho,
                              d.L2, d.delta, gscale, gvol.as<float>(), gpw.as<float>(), contrib.as<double>(),
                              rows.as<double>(), st));
    std::vector<double> r((size_t)n * H);
    int e = 0, te = 0;
    CNNCRF_CUDA(cudaMemcpyAsync(r.data(), rows.get(), sizeof(double) * r.size(), cudaMemcpyDeviceToHost, st));
    CNNCRF_CUDA(cudaMemcpyAsync(&e, err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    CNNCRF_CUDA(cudaMemcpyAsync(&te, tcerr.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    CNNCRF_CUDA(cudaStreamSynchronize(st));
    if (te) {
        CNNCRF_CUDA(cudaMemset(tcerr.get(), 0, sizeof(int)));
        return fail(CNNCRF_ETIMEOUT, "train: a tensor-core kernel gave up on a bounded wait");
    }
    if (e) return fail(CNNCRF_EINVAL, "train: %d ground-truth labels outside 0..%d", e, D - 1);
    if (loss)
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int y = 0; y < H; ++y) s += r[(size_t)i * H + y];
            loss[i] = d.mean_loss ? s / ((double)H * W) : s;
        }
    if (yh_out)
        CNNCRF_CUDA(cudaMemcpyAsync(yh_out, labels.get(), sizeof(int32_t) * N, cudaMemcpyDeviceToDevice, st));
    hinged = true;
    return CNNCRF_OK;
}

// nimg: the batch's images (both sides' for a feature layer).
// dz: the layer's output gradient (dense FP32), turned into the pre-activation
// gradient in place; y: the layer's output at channel stride ys; dprev (if
// set): the input gradient (dense FP32).  ready: on entry, whether dz already
// holds the output gradient times 1 - y^2 with its BF16 padded copy in
// dpad[dcur] (the layer above's fused input gradient made them); on exit,
// whether this call made dprev so for `below`, the layer whose output is `in`.
int cnncrf_train::layer_back(TLayer &L, int nimg, const void *in, bool in_bf16, long in_pix, long in_row,
                             long in_img, const void *y, int ys, float *dz, float *dprev, bool &ready,
                             const TLayer *below)
{
    const int Ho = L.hout(), Wo = L.wout();
    const int ph = L.kh - 1, pwd = L.kw - 1;
    const bool tcd = dprev && L.w16d.get(); // the input gradient on the tensor cores (BF16 mode)
    if (!ready) {
        if (tcd || L.tcw) // dz and its BF16 padded copy, the tensor-core operand
            CNNCRF_TRY(k::train_tanh_bwd_pad(dz, y, nimg, Ho, Wo, L.cout, ys, ph, pwd, pad_to(L.cout, 64),
                                             dpad[dcur].get(), st));
        else
            CNNCRF_TRY(k::train_tanh_bwd(dz, y, bf16, (long)nimg * Ho * Wo, L.cout, ys, st));
    }
    const bool was_ready = ready;
    ready = false;
    if (L.tcw && in_bf16) { // BF16 mode, tensor cores
        CNNCRF_TRY(k::wgrad_tc(dpad[dcur].get(), L.cout, pad_to(L.cout, 64), in, in_pix, in_row, in_img, L.cin, L.kh,
                               L.kw, nimg, Ho, Wo, wgs.get(), wgs_bytes, gradp(L.wslot), tcerr.as<int>(), st));
        if (L.bslot >= 0) {
            if (was_ready && bias_ready) // the sums the layer above's fused epilogue left
                CNNCRF_TRY(k::train_bias_reduce(bpart.as<float>(), bsplits, L.cout, gradp(L.bslot), st));
            else
                CNNCRF_TRY(k::train_bias_grad(dz, L.cout, (long)nimg * Ho * Wo, partb.as<float>(), gradp(L.bslot), st));
        }
    } else {
        CNNCRF_TRY(k::train_wgrad(dz, L.cout, in, in_bf16, in_pix, in_row, in_img, L.cin, L.kh, L.kw, nimg, Ho, Wo,
                                  part.as<float>(), gradp(L.wslot), L.bslot >= 0 ? gradp(L.bslot) : nullptr,
                                  partb.as<float>(), st));
    }
    if (!dprev) return CNNCRF_OK;
    if (tcd) { // dprev = the valid convolution of the padded dz with the unflipped, transposed kernel
        k::TcConvArgs t{};
        t.in = dpad[dcur].get(), t.n_img = nimg, t.Hin = Ho + 2 * ph, t.Win = Wo + 2 * pwd;
        t.cp_in = pad_to(L.cout, 64), t.cin = L.cout;
        t.wt = L.w16d.get(), t.np = umma_n(L.cin), t.cout = L.cin, t.kh = L.kh, t.kw = L.kw;
        t.mode = 3, t.out = dprev, t.cp_out = L.cin, t.err = tcerr.as<int>();
        // fused with the layer below's tanh backward when its gradients read the padded copy too
        const bool fuse = below && in_bf16 && (below->tcw || below->w16d.get()) && below->hout() == L.hin &&
                          below->wout() == L.win && below->cout == L.cin && in_row == (long)L.win * in_pix &&
                          in_img == (long)L.hin * in_row;
        bias_ready = false;
        if (fuse) {
            const int bph = below->kh - 1, bpw = below->kw - 1, bcp = pad_to(below->cout, 64);
            CNNCRF_TRY(k::train_zero_border(dpad[dcur ^ 1].get(), nimg, L.hin, L.win, bcp, bph, bpw, st));
            t.mode = 4, t.aux = in, t.aux_cs = (int)in_pix;
            t.out16 = dpad[dcur ^ 1].get(), t.o16_cs = bcp, t.o16_ph = bph, t.o16_pw = bpw;
            // the FP32 dz only where a CUDA-core gradient of the layer below reads it
            if (below->tcw && (!below->dprev || below->w16d.get())) t.out = nullptr;
            if (below->bslot >= 0 && below->tcw) t.bias_part = bpart.as<float>(), t.bias_splits = &bsplits;
        }
        CNNCRF_TRY(k::conv_tc(t, st));
        if (fuse) dcur ^= 1, ready = true, bias_ready = t.bias_part != nullptr;
        return CNNCRF_OK;
    }
    CNNCRF_TRY(k::train_pad_zero(dz, nimg, Ho, Wo, L.cout, ph, pwd, padb.as<float>(), st));
    const int Hp = Ho + 2 * ph, Wp = Wo + 2 * pwd;
    k::ConvArgs a{padb.as<float>(), Hp, Wp, L.cout, (long)L.cout, (long)Wp * L.cout, L.wd.as<float>(), nullptr,
                  L.cin, L.kh, L.kw, 0, dprev};
    a.n_img = nimg, a.in_img = (long)Hp * Wp * L.cout, a.out_img = (long)L.hin * L.win * L.cin;
    return k::conv_simt(a, st);
}

int cnncrf_train::backward(const float *gv, const float *gp)
{
    if (!forwarded) return fail(CNNCRF_ESTATE, "train: backward before forward");
    if (!gv && !hinged) return fail(CNNCRF_ESTATE, "train: backward from the hinge before hinge");
    if (!gv) gv = gvol.as<float>(), gp = gpw.as<float>();
    const int F = d.feat_channels, P = d.pw_channels, L = (int)feat.size(), fs = fstride(), ps = pstride();
    const long N = (long)n * H * W;
    CNNCRF_CUDA(cudaMemsetAsync(grad.get(), 0, total * sizeof(float), st));
    if (tc_corr)
        CNNCRF_TRY(k::corr_bwd_tc(fside(0), fside(1), fs, gv, dlist.as<float>(), n, H, W, F, D, omin, omax, df_s(0),
                                  df_s(1), tcerr.as<int>(), st));
    else
        CNNCRF_TRY(k::train_corr_bwd(fside(0), fside(1), bf16, fs, gv, dlist.as<float>(), n, H, W, F, D, omin,
                                     omax, df_s(0), df_s(1), st));
    // the feature net, both sides at once: each weight gradient sums the two sides in one launch
    float *cur = dy.as<float>(), *nxt = dyb.as<float>();
    bool ready = false;
    TLayer &top_l = feat[L - 1];
    if (bf16 && top_l.tcw && top_l.w16d.get() && fs == 128 && top_l.kh == top_l.kw) {
        // the normalisation's adjoint, tanh', the padded copy and the bias sums in one pass
        CNNCRF_TRY(k::train_l2norm_tanh_bwd_pad(actp(L - 1), fs, df.as<float>(), nf(), H, W, F, top_l.kh - 1,
                                                top_l.kw - 1, dpad[dcur].get(), bpart.as<float>(), &bsplits, st));
        ready = bias_ready = true;
    } else {
        CNNCRF_TRY(k::train_l2norm_bwd(actp(L - 1), bf16, fs, df.as<float>(), 2 * N, F, dy.as<float>(), st));
    }
    int top = L - 1;
    while (top >= 0) {
        int c = top - 1; // the checkpoint under this segment (-1: the normalised input)
        while (c >= 0 && !keep[c]) --c;
        for (int j = c + 1; j < top; ++j) CNNCRF_TRY(run_layer(j)); // recompute the segment
        for (int j = top; j > c; --j) {
            TLayer &Ly = feat[j];
            // the first layer reads the normalised input: its BF16 copy for the tensor-core weight gradient
            const bool n16 = j == 0 && Ly.tcw;
            const void *in = j > 0 ? actp(j - 1) : n16 ? norm16.get() : (const void *)norm.get();
            const bool ib = (j > 0 && bf16) || n16;
            const int cs = j > 0 ? fs : n16 ? 64 : ic;
            CNNCRF_TRY(layer_back(Ly, nf(), in, ib, cs, (long)Ly.win * cs, (long)Ly.hin * Ly.win * cs, actp(j), fs,
                                  cur, j > 0 ? nxt : nullptr, ready, j > 0 ? &feat[j - 1] : nullptr));
            std::swap(cur, nxt);
        }
        top = c;
    }
    if (gp) {
        // head: gh = gpw sign(h), dy2 = W^T gh; its weight gradient is a 1x1 wgrad on y2
        ready = false;
        if (bf16 && pw[1].tcw && pw[1].w16d.get() && ps == 64 && P <= 64) {
            // with the second pairwise layer's tanh', padded copy and bias sums
            CNNCRF_TRY(k::train_head_tanh_bwd_pad(y2.get(), ps, param(pw[2].wslot), gp, n, H, W, P, pw[1].kh - 1,
                                                  pw[1].kw - 1, gh.as<float>(), dpad[dcur].get(), bpart.as<float>(),
                                                  &bsplits, st));
            ready = bias_ready = true;
        } else {
            CNNCRF_TRY(k::train_head_bwd(y2.get(), bf16, ps, param(pw[2].wslot), gp, n, H * W, P, gh.as<float>(),
                                         dy.as<float>(), st));
        }
        CNNCRF_TRY(k::train_wgrad_head(gh.as<float>(), y2.get(), bf16, ps, (long)n * H * W, P, partb.as<float>(),
                                       gradp(pw[2].wslot), st));
        CNNCRF_TRY(layer_back(pw[1], n, y1.get(), bf16, ps, (long)(W + 2) * ps, (long)(H + 2) * (W + 2) * ps, y2.get(),
                              ps, dy.as<float>(), dyb.as<float>(), ready, &pw[0]));
        const int cr = p - 2;
        if (pw[0].tcw) {
            const void *in = (const char *)norm16.get() + 2 * ((size_t)cr * w + cr) * 64;
            CNNCRF_TRY(layer_back(pw[0], n, in, true, 64, (long)w * 64, (long)h * w * 64, y1.get(), ps, dyb.as<float>(),
                                  nullptr, ready, nullptr));
        } else {
            const float *in = norm_s(0) + ((size_t)cr * w + cr) * ic;
            CNNCRF_TRY(layer_back(pw[0], n, in, false, ic, (long)w * ic, (long)h * w * ic, y1.get(), ps,
                                  dyb.as<float>(), nullptr, ready, nullptr));
        }
    }
    return CNNCRF_OK;
}

// ---------------------------------------------------------------- C ABI

extern "C" {

int cnncrf_train_default_desc(cnncrf_train_desc *d)
{
    if (!d) return fail(CNNCRF_EINVAL, "null argument");
    std::memset(d, 0, sizeof *d);
    d->num_layers = 7;
    d->topology = CNNCRF_TOPO_ALL3X3;
    d->feat_channels = 100;
    d->pw_channels = 64;
    d->disp_min = 0.0f, d->disp_step = 1.0f, d->disp_max = 127.0f;
    d->lambda = 1.0f;
    d->L1 = 0.5f, d->L2 = 1.5f, d->delta = 3;
    d->crf_shape = CNNCRF_RHO_LINEAR;
    d->crf_slack = 0.5f;
    d->crf_iters = 8;
    d->mean_loss = 1;
    d->precision = CNNCRF_BF16;
    d->checkpoint_every = 3;
    d->tc_wgrad = 1;
    d->tc_dgrad = 1;
    return CNNCRF_OK;
}

int cnncrf_train_create(cnncrf_train_t *out, const cnncrf_train_desc *desc, int npairs, int width, int height)
{
    clear_error();
    if (!out || !desc) return fail(CNNCRF_EINVAL, "null argument");
    *out = nullptr;
    const cnncrf_train_desc &d = *desc;
    if (npairs < 1 || width < 1 || height < 1) return fail(CNNCRF_EINVAL, "train: bad size");
    if (d.num_layers < 1 || d.num_layers > 16) return fail(CNNCRF_EINVAL, "train: num_layers %d", d.num_layers);
    if (d.topology != CNNCRF_TOPO_REF && d.topology != CNNCRF_TOPO_ALL3X3)
        return fail(CNNCRF_EINVAL, "train: topology %d", d.topology);
    if (d.feat_channels < 1 || d.feat_channels > 128 || d.pw_channels < 1 || d.pw_channels > 128)
        return fail(CNNCRF_EINVAL, "train: channels %d / %d outside 1..128", d.feat_channels, d.pw_channels);
    if (d.precision != CNNCRF_FP32 && d.precision != CNNCRF_BF16) return fail(CNNCRF_EINVAL, "train: precision");
    if (d.checkpoint_every < 0) return fail(CNNCRF_EINVAL, "train: checkpoint_every %d", d.checkpoint_every);
    if (!(d.disp_step > 0.0f) || d.delta < 1 || d.delta > 4 || d.crf_iters < 1 || !(d.crf_slack > 0.0f) ||
        d.crf_slack > 1.0f)
        return fail(CNNCRF_EINVAL, "train: bad disparity step or CRF options");
    auto *t = new cnncrf_train;
    t->d = d;
    t->n = npairs, t->W = width, t->H = height;
    int rc = t->build();
    if (rc != CNNCRF_OK) {
        delete t;
        return rc;
    }
    *out = t;
    return CNNCRF_OK;
}

int cnncrf_train_destroy(cnncrf_train_t t)
{
    if (t) cudaDeviceSynchronize();
    delete t;
    return CNNCRF_OK;
}

int cnncrf_train_set_stream(cnncrf_train_t t, cnncrf_stream_t stream)
{
    if (!t) return fail(CNNCRF_EINVAL, "null train");
    t->st = (cudaStream_t)stream;
    return CNNCRF_OK;
}

int cnncrf_train_num_params(cnncrf_train_t t, int *n)
{
    if (!t || !n) return fail(CNNCRF_EINVAL, "null argument");
    *n = (int)t->off.size();
    return CNNCRF_OK;
}

int cnncrf_train_param_shape(cnncrf_train_t t, int i, int64_t shape[4], int *ndim)
{
    if (!t || !shape || !ndim) return fail(CNNCRF_EINVAL, "null argument");
    for (auto *v : {&t->feat, &t->pw})
        for (auto &L : *v) {
            if (L.wslot == i) {
                shape[0] = L.cout, shape[1] = L.cin, shape[2] = L.kh, shape[3] = L.kw;
                *ndim = 4;
                return CNNCRF_OK;
            }
            if (L.bslot == i) {
                shape[0] = L.cout;
                *ndim = 1;
                return CNNCRF_OK;
            }
        }
    return fail(CNNCRF_EINVAL, "train: parameter %d outside 0..%zu", i, t->off.size() - 1);
}

int cnncrf_train_init_xavier(cnncrf_train_t t, uint64_t seed)
{
    clear_error();
    if (!t) return fail(CNNCRF_EINVAL, "null train");
    std::vector<float> all(t->total, 0.0f);
    for (size_t i = 0; i < t->off.size(); ++i) {
        int64_t s[4];
        int nd;
        CNNCRF_TRY(cnncrf_train_param_shape(t, (int)i, s, &nd));
        if (nd == 4) cnncrf_xavier_fill(all.data() + t->off[i], (int)s[0], (int)s[1], (int)s[2], (int)s[3], seed, (int)i);
    }
    CNNCRF_CUDA(cudaMemcpy(t->theta.get(), all.data(), t->total * sizeof(float), cudaMemcpyHostToDevice));
    CNNCRF_CUDA(cudaMemset(t->vel.get(), 0, t->total * sizeof(float)));
    CNNCRF_TRY(t->refresh());
    t->forwarded = t->hinged = false;
    return CNNCRF_OK;
}

static int slot_check(cnncrf_train_t t, int i, const void *data, size_t count)
{
    if (!t || !data) return fail(CNNCRF_EINVAL, "null argument");
    if (i < 0 || i >= (int)t->off.size()) return fail(CNNCRF_EINVAL, "train: parameter %d", i);
    if (count != t->cnt[i]) return fail(CNNCRF_ESHAPE, "train: parameter %d has %zu values, not %zu", i, t->cnt[i], count);
    return CNNCRF_OK;
}

int cnncrf_train_set_param(cnncrf_train_t t, int i, const float *data, size_t count)
{
    clear_error();
    CNNCRF_TRY(slot_check(t, i, data, count));
    CNNCRF_CUDA(cudaStreamSynchronize(t->st));
    CNNCRF_CUDA(cudaMemcpy(t->param(i), data, count * sizeof(float), cudaMemcpyDefault));
    CNNCRF_TRY(t->refresh());
    t->forwarded = t->hinged = false;
    return CNNCRF_OK;
}

int cnncrf_train_get_param(cnncrf_train_t t, int i, float *data, size_t count)
{
    clear_error();
    CNNCRF_TRY(slot_check(t, i, data, count));
    CNNCRF_CUDA(cudaStreamSynchronize(t->st));
    CNNCRF_CUDA(cudaMemcpy(data, t->param(i), count * sizeof(float), cudaMemcpyDefault));
    return CNNCRF_OK;
}

int cnncrf_train_get_grad(cnncrf_train_t t, int i, float *data, size_t count)
{
    clear_error();
    CNNCRF_TRY(slot_check(t, i, data, count));
    CNNCRF_CUDA(cudaStreamSynchronize(t->st));
    CNNCRF_CUDA(cudaMemcpy(data, t->gradp(i), count * sizeof(float), cudaMemcpyDefault));
    return CNNCRF_OK;
}

int cnncrf_train_forward(cnncrf_train_t t, const float *d_left, const float *d_right)
{
    CNNCRF_RANGE("train_forward");
    clear_error();
    if (!t || !d_left || !d_right) return fail(CNNCRF_EINVAL, "null argument");
    return t->forward(d_left, d_right);
}

int cnncrf_train_outputs(cnncrf_train_t t, const float **d_volume, const float **d_pairwise, int *depth)
{
    if (!t) return fail(CNNCRF_EINVAL, "null train");
    if (!t->forwarded) return fail(CNNCRF_ESTATE, "train: outputs before forward");
    if (d_volume) *d_volume = t->vol.as<float>();
    if (d_pairwise) *d_pairwise = t->pwout.as<float>();
    if (depth) *depth = t->D;
    return CNNCRF_OK;
}

int cnncrf_train_hinge(cnncrf_train_t t, const int32_t *d_gt, double *h_loss, int32_t *d_labels)
{
    CNNCRF_RANGE("train_hinge");
    clear_error();
    if (!t || !d_gt) return fail(CNNCRF_EINVAL, "null argument");
    return t->hinge(d_gt, h_loss, d_labels);
}

int cnncrf_train_autotune(cnncrf_train_t t)
{
    clear_error();
    if (!t) return fail(CNNCRF_EINVAL, "null train");
    if (!t->forwarded) return fail(CNNCRF_ESTATE, "train: autotune before forward");
    const long N = (long)t->n * t->H * t->W, img = (long)t->H * t->W;
    // the hinge's problem: the unary and lambda times the pairwise output, all crops in one solve
    CNNCRF_CUDA(cudaMemcpyAsync(t->wts.get(), t->pwout.get(), sizeof(float) * N * 2, cudaMemcpyDeviceToDevice, t->st));
    CNNCRF_TRY(k::scale(t->wts.as<float>(), N * 2, t->d.lambda, t->st));
    k::CrfParams cp;
    cp.L1 = t->d.L1, cp.L2 = t->d.L2, cp.delta = t->d.delta, cp.shape = t->d.crf_shape, cp.slack = t->d.crf_slack;
    return k::crf_autotune(t->vol.as<float>(), t->wts.as<float>(), t->wts.as<float>() + img, 2 * img, t->W, t->H,
                           t->D, t->n, cp, t->crfws.get(), t->crfws_bytes, t->st, true);
}

int cnncrf_train_hinge_grads(cnncrf_train_t t, const float **d_gvol, const float **d_gpw)
{
    if (!t) return fail(CNNCRF_EINVAL, "null train");
    if (!t->hinged) return fail(CNNCRF_ESTATE, "train: hinge gradients before hinge");
    if (d_gvol) *d_gvol = t->gvol.as<float>();
    if (d_gpw) *d_gpw = t->gpw.as<float>();
    return CNNCRF_OK;
}

int cnncrf_train_backward(cnncrf_train_t t, const float *d_gvol, const float *d_gpw)
{
    CNNCRF_RANGE("train_backward");
    clear_error();
    if (!t) return fail(CNNCRF_EINVAL, "null train");
    if (!d_gvol && d_gpw) return fail(CNNCRF_EINVAL, "train: pairwise gradient without a volume gradient");
    return t->backward(d_gvol, d_gpw);
}

int cnncrf_train_sgd(cnncrf_train_t t, float lr, float momentum)
{
    CNNCRF_RANGE("train_sgd");
    clear_error();
    if (!t) return fail(CNNCRF_EINVAL, "null train");
    if (!(lr >= 0.0f) || !(momentum >= 0.0f) || momentum >= 1.0f)
        return fail(CNNCRF_EINVAL, "train: lr %g, momentum %g", lr, momentum);
    CNNCRF_TRY(k::train_sgd(t->theta.as<float>(), t->grad.as<float>(), t->vel.as<float>(), (long)t->total, lr,
                            momentum, t->st));
    CNNCRF_TRY(t->refresh());
    t->forwarded = t->hinged = false;
    return CNNCRF_OK;
}

// Checkpoints: the master weights as arr_i (the parameter-file layout) and
// the momentum as mom_i, both copied through one host staging array.
int cnncrf_train_save(cnncrf_train_t t, const char *npz_path)
{
    clear_error();
    if (!t || !npz_path) return fail(CNNCRF_EINVAL, "null argument");
    CNNCRF_CUDA(cudaStreamSynchronize(t->st));
    std::vector<float> w(t->total), v(t->total);
    CNNCRF_CUDA(cudaMemcpy(w.data(), t->theta.get(), t->total * sizeof(float), cudaMemcpyDeviceToHost));
    CNNCRF_CUDA(cudaMemcpy(v.data(), t->vel.get(), t->total * sizeof(float), cudaMemcpyDeviceToHost));
    const int n = (int)t->off.size();
    std::vector<NpzMember> m;
    for (int pass = 0; pass < 2; ++pass)
        for (int i = 0; i < n; ++i) {
            int64_t s[4];
            int nd = 0;
            CNNCRF_TRY(cnncrf_train_param_shape(t, i, s, &nd));
            NpzMember a;
            a.key = (pass == 0 ? "arr_" : "mom_") + std::to_string(i);
            a.data = (pass == 0 ? w.data() : v.data()) + t->off[i];
            a.shape.assign(s, s + nd);
            m.push_back(std::move(a));
        }
    return npz_save(npz_path, m);
}

int cnncrf_train_load(cnncrf_train_t t, const char *npz_path)
{
    clear_error();
    if (!t || !npz_path) return fail(CNNCRF_EINVAL, "null argument");
    std::vector<float> w(t->total), v(t->total, 0.0f);
    const int n = (int)t->off.size();
    for (int i = 0; i < n; ++i) {
        int64_t s[4];
        int nd = 0;
        CNNCRF_TRY(cnncrf_train_param_shape(t, i, s, &nd));
        NpyArray a;
        CNNCRF_TRY(npz_load(npz_path, "arr_" + std::to_string(i), &a));
        if (a.shape != std::vector<int64_t>(s, s + nd) || a.data.size() != t->cnt[i])
            return fail(CNNCRF_ESHAPE, "train_load: %s: arr_%d does not have the slot's shape", npz_path, i);
        std::memcpy(w.data() + t->off[i], a.data.data(), t->cnt[i] * sizeof(float));
        // the momentum is optional: a plain parameter file has none
        NpyArray mo;
        if (npz_load(npz_path, "mom_" + std::to_string(i), &mo) == CNNCRF_OK) {
            if (mo.shape != a.shape)
                return fail(CNNCRF_ESHAPE, "train_load: %s: mom_%d does not have the slot's shape", npz_path, i);
            std::memcpy(v.data() + t->off[i], mo.data.data(), t->cnt[i] * sizeof(float));
        }
    }
    clear_error(); // the absent mom_i lookups above are not errors
    CNNCRF_CUDA(cudaStreamSynchronize(t->st));
    CNNCRF_CUDA(cudaMemcpy(t->theta.get(), w.data(), t->total * sizeof(float), cudaMemcpyHostToDevice));
    CNNCRF_CUDA(cudaMemcpy(t->vel.get(), v.data(), t->total * sizeof(float), cudaMemcpyHostToDevice));
    CNNCRF_TRY(t->refresh());
    t->forwarded = t->hinged = false;
    return CNNCRF_OK;
}

int cnncrf_train_step(cnncrf_train_t t, const float *d_left, const float *d_right, const int32_t *d_gt, float lr,
                      float momentum, double *h_loss)
{
    CNNCRF_RANGE("train_step");
    clear_error();
    if (!t || !d_left || !d_right || !d_gt) return fail(CNNCRF_EINVAL, "null argument");
    CNNCRF_TRY(t->forward(d_left, d_right));
    CNNCRF_TRY(t->hinge(d_gt, h_loss, nullptr));
    CNNCRF_TRY(t->backward(nullptr, nullptr));
    return cnncrf_train_sgd(t, lr, momentum);
}

} // extern "C"
