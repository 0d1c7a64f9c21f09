// net.h -- the StereoNet / ColorStereoNet object behind cnncrf_net_t.
#pragma once

#include <vector>

#include "common.h"
#include "kernels.h"

struct cnncrf_net {
    struct Layer {
        int cin, cout, kh, kw, act, wslot, bslot;
        cnncrf::DevBuf wt;   // FP32 [K][128] flipped / transposed / padded
        cnncrf::DevBuf bias; // FP32 [128]
        cnncrf::DevBuf wt16; // BF16 [Npad][taps][Cpad] K-major, for the tensor-core path
    };

    cnncrf_net_desc d{};
    int n = 1, h = 0, w = 0, pad = 0, H = 0, W = 0;
    cudaStream_t st = nullptr;
    std::vector<Layer> feat, pw;
    std::vector<std::vector<float>> host;
    std::vector<char> have;

    // disparities (StereoCorrelation state)
    std::vector<float> list;
    cnncrf::DevBuf d_list;
    int D = 0;
    bool interp = false, force_interp = false;
    bool int_list = false; // every stored disparity an exact integer
    int omin = 0, omax = 0;
    float *vol = nullptr;
    cnncrf::DevBuf vol_own;
    float *pwout = nullptr;
    cnncrf::DevBuf pw_own;
    // BF16 path: an owner-supplied buffer for the volume's 16-bit fixed-point
    // copy (the CRF's unary); volq_valid after a predict that wrote it (the
    // tensor-core correlation writes it; its SIMT fallback does not).  With
    // volq set and vol_fp32 false the FP32 volume is not written when the copy is.
    void *volq = nullptr;
    bool volq_valid = false;
    bool vol_fp32 = true;

    // activations
    cnncrf::DevBuf norm[2], act[2][2], pwa, pwb, scratch;
    float *feats[2] = {nullptr, nullptr};
    bool inited = false;
    // the concatenating topology: growth rate g, the zero-bordered input
    // [n][h+2][w+2][ic] and features [n][h+2][w+2][g L] of each side, and
    // the features cropped to [n][H][W][g L] for the correlation
    int growth = 0;
    cnncrf::DevBuf cx[2], cz[2], cf[2];
    int predict_concat(const float *left, const float *right);

    // tensor-core path: BF16 NHWC activations of both images, channel
    // padded to cp_feat (feature net) / cp_pw (pairwise net)
    int np_feat = 0, cp_feat = 0, np_pw = 0, cp_pw = 0;
    cnncrf::DevBuf a16[2], pw16, head16, err;
    const void *feat16 = nullptr; // [2][H][W][cp_feat] after predict
    int alloc_bf16();
    int check_error();
    // the tensor-core convolutions of the last BF16 predict, for autotune_conv
    std::vector<cnncrf::k::TcConvArgs> tc_calls;
    // time every launch form of those convolutions and enter the fastest in
    // the process-wide conv tuning table (synchronises; rewrites the outputs)
    int autotune_conv();

    int num_params() const { return (int)host.size(); }
    int expected_shape(int i, int64_t s[4], int *nd) const;
    int upload(int slot);
    int predict(const float *left, const float *right);
    int predict_fp32(const float *left, const float *right, bool reuse_left);
    // FP32 path: the next predict's left input is the last predict's (same
    // padded image): keep its left features (and normalised image) instead of
    // recomputing them.  One-shot; honoured only while left_ok.
    bool reuse_left = false;
    bool left_ok = false; // feats[0] / norm[0] are those of the last completed FP32 predict
    int predict_bf16(const float *left, const float *right);
    int pairwise_fp32();
    int set_disparities(float mn, float mx, float step, float *d_out);
};

namespace cnncrf {
// ConcatStereoNet's growth rate for a depth (stereo/concatstereonet.cpp:28-56); 0 for any other depth
int concat_growth(int layers);
// mirror padding a net of this description needs around its images
// (stereo/stereo.cpp:204-217): the receptive-field loss / 2, 0 for the concatenating net
int net_padding(const cnncrf_net_desc &d);
} // namespace cnncrf
