// net_bf16.cu -- ColorStereoNet::predict on the tensor cores: the BF16 path.
//
//   normalise (FP32, as the exact path)
//   layer 1          tcgen05 conv with the patch gathered per pixel (K =
//                    9 * Cin <= 45 is too thin for TMA k-blocks), BF16
//                    inputs and weights, BF16 NHWC output padded to cp_feat
//   layers 2..L      tcgen05 implicit GEMM over both images at once; the last
//                    layer L2-normalises in its epilogue for the 1-<fL,fR> unary
//   correlation      BF16 features, FP32 accumulation, unary fused: tcgen05
//                    banded GEMM for integer lists of band <= 128, SIMT
//                    banded kernel otherwise (fractional or wide lists)
//   pairwise net     tcgen05 3x3 (3 -> 64, gathered patch) into BF16, then tcgen05 3x3 (64 -> 64)
//                    whose epilogue applies the 1x1 head and |.| and writes wx, wy
// Reference: stereo/stereonet.cpp:250-421, stereo/colorstereonet.cpp:38-77.
#include "kernels.h"
#include "net.h"

using namespace cnncrf;

namespace {
int pad_to(int c, int m) { return (c + m - 1) / m * m; }
int umma_n(int cout) { return cout <= 64 ? 64 : (cout <= 112 ? 112 : 128); }
} // namespace

int cnncrf_net::alloc_bf16()
{
    cp_feat = pad_to(d.feat_channels, 64);
    np_feat = umma_n(d.feat_channels);
    size_t h1 = h - 2, w1 = w - 2; // layer-1 output, the largest activation
    size_t bytes = 2 * (size_t)n * h1 * w1 * cp_feat * 2; // [side][pair][h][w][cp] BF16
    for (int i = 0; i < 2; ++i) {
        CNNCRF_TRY(a16[i].reserve(bytes));
        // channels past feat_channels are never written and must read as zero
        CNNCRF_CUDA(cudaMemset(a16[i].get(), 0, bytes));
    }
    if (d.with_pairwise) {
        cp_pw = pad_to(d.pw_channels, 64);
        np_pw = umma_n(d.pw_channels);
        size_t pb = (size_t)n * (H + 2) * (W + 2) * cp_pw * 2;
        CNNCRF_TRY(pw16.reserve(pb));
        CNNCRF_CUDA(cudaMemset(pw16.get(), 0, pb));
    }
    CNNCRF_TRY(err.reserve(sizeof(int)));
    CNNCRF_CUDA(cudaMemset(err.get(), 0, sizeof(int)));
    return CNNCRF_OK;
}

int cnncrf_net::check_error()
{
    if (d.precision != CNNCRF_BF16 || !err.get()) return CNNCRF_OK;
    int e = 0;
    CNNCRF_CUDA(cudaMemcpyAsync(&e, err.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    CNNCRF_CUDA(cudaStreamSynchronize(st));
    if (e) {
        CNNCRF_CUDA(cudaMemsetAsync(err.get(), 0, sizeof(int), st));
        return fail(CNNCRF_ETIMEOUT, "a tensor-core kernel gave up on a bounded wait");
    }
    return CNNCRF_OK;
}

int cnncrf_net::predict_bf16(const float *left, const float *right)
{
    tc_calls.clear();
    if (d.num_layers < 2) return fail(CNNCRF_EUNSUPPORTED, "BF16 path needs >= 2 feature layers");
    const float *img[2] = {left, right};
    const int ic = d.in_channels, F = d.feat_channels, cp = cp_feat;
    const size_t h1 = h - 2, w1 = w - 2;
    for (int s = 0; s < 2; ++s) {
        CNNCRF_TRY(k::normalize(img[s], w, h, ic, norm[s].as<float>(), scratch.get(), st, n));
        Layer &L0 = feat[0];
        k::ConvArgs a{norm[s].as<float>(), h, w, ic, (long)ic, (long)w * ic, L0.wt.as<float>(), L0.bias.as<float>(),
                      F, 3, 3, 1, nullptr};
        a.out16 = (uint16_t *)a16[0].get() + (size_t)s * n * h1 * w1 * cp;
        a.out_cs = cp;
        a.n_img = n, a.in_img = (long)h * w * ic, a.out_img = (long)(h1 * w1 * cp);
        if (k::conv_first_tc_supported(a)) CNNCRF_TRY(k::conv_first_tc(a, err.as<int>(), st));
        else CNNCRF_TRY(k::conv_simt(a, st));
    }
    int hin = (int)h1, win = (int)w1;
    int cur = 0;
    for (size_t l = 1; l < feat.size(); ++l) {
        Layer &L = feat[l];
        k::TcConvArgs t{};
        t.in = a16[cur].get();
        t.n_img = 2 * n, t.Hin = hin, t.Win = win, t.cp_in = cp, t.cin = F; // left images, then right images
        t.wt = L.wt16.get();
        t.np = np_feat, t.cout = F, t.kh = L.kh, t.kw = L.kw;
        t.bias = L.bias.as<float>();
        t.head = nullptr;
        t.mode = (l + 1 == feat.size() && d.unary == CNNCRF_UNARY_ONE_MINUS_DOT) ? 1 : 0;
        t.out = a16[cur ^ 1].get();
        t.cp_out = cp;
        t.err = err.as<int>();
        CNNCRF_TRY(k::conv_tc(t, st));
        tc_calls.push_back(t);
        hin -= L.kh - 1, win -= L.kw - 1;
        cur ^= 1;
    }
    if (hin != H || win != W) return fail(CNNCRF_ESHAPE, "BF16 feature map %dx%d != %dx%d", win, hin, W, H);
    const uint16_t *f = (const uint16_t *)a16[cur].get();
    const size_t fimg = (size_t)H * W * cp;
    feat16 = f;
    const bool ip = interp || force_interp;
    volq_valid = false;
    k::UnaryQ16 uq;
    if (!ip && int_list && k::corr_tc_supported(F, cp, list.data(), D, d.unary)) {
        void *q = (volq && k::unary_q16(d.unary, &uq)) ? volq : nullptr;
        CNNCRF_TRY(k::correlation_tc(f, n, H, W, F, cp, d_list.as<float>(), list.data(), D, d.unary,
                                     (q && !vol_fp32) ? nullptr : vol, err.as<int>(), st, q));
        volq_valid = q != nullptr;
    } else {
        CNNCRF_TRY(k::correlation_bf16(f, f + (size_t)n * fimg, H, W, F, cp, d_list.as<float>(), D, omin, omax, ip,
                                       d.unary, vol, st, n, (long)fimg));
    }
    if (d.with_pairwise) {
        int cr = pad - 2;
        const float *in = norm[0].as<float>() + ((size_t)cr * w + cr) * ic;
        k::ConvArgs a1{in, H + 4, W + 4, pw[0].cin, (long)ic, (long)w * ic, pw[0].wt.as<float>(), pw[0].bias.as<float>(),
                       pw[0].cout, 3, 3, 1, nullptr};
        a1.out16 = pw16.get();
        a1.out_cs = cp_pw;
        a1.n_img = n, a1.in_img = (long)h * w * ic, a1.out_img = (long)(H + 2) * (W + 2) * cp_pw;
        if (k::conv_first_tc_supported(a1)) CNNCRF_TRY(k::conv_first_tc(a1, err.as<int>(), st));
        else CNNCRF_TRY(k::conv_simt(a1, st));
        k::TcConvArgs t{};
        t.in = pw16.get();
        t.n_img = n, t.Hin = H + 2, t.Win = W + 2, t.cp_in = cp_pw, t.cin = pw[1].cin;
        t.wt = pw[1].wt16.get();
        t.np = np_pw, t.cout = pw[1].cout, t.kh = 3, t.kw = 3;
        t.bias = pw[1].bias.as<float>();
        t.head = head16.as<float>();
        t.mode = 2;
        t.out = pwout;
        t.cp_out = 0;
        t.err = err.as<int>();
        CNNCRF_TRY(k::conv_tc(t, st));
        tc_calls.push_back(t);
    }
    return CNNCRF_OK;
}

int cnncrf_net::autotune_conv()
{
    if (d.precision != CNNCRF_BF16) return CNNCRF_OK;
    for (const auto &t : tc_calls) CNNCRF_TRY(cnncrf::k::conv_tc_autotune(t, st));
    return check_error();
}
