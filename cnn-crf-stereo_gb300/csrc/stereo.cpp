// stereo.cpp -- the Stereo orchestrator behind cnncrf_stereo_t: buffers,
// lazy net construction, the CRF call, label remap and the TV/Huber
// refinement, all enqueued on one stream.
//
// Reference: stereo/stereo.cpp (initialize 64-105, setColorImages 117-126,
// computeSlackPropagation 129-162, computeArgMax 164-177, computeVolume
// 179-318, fuseTHuberQuadFit 388-404) and cuda::fuseTHuberQuadFit
// (stereo/stereo.cu:1113-1170).
#include <cmath>
#include <string>
#include <vector>

#include "common.h"
#include "kernels.h"
#include "net.h"

using namespace cnncrf;

struct cnncrf_stereo {
    cnncrf_stereo_options o{};
    cudaStream_t st = nullptr;
    int W = 0, H = 0, depth = 0;
    float dmin = 0, dstep = 1, dmax = 0;
    bool inited = false;
    int matching = CNNCRF_MATCH_CENSUS;
    int num_layers = 3; // stereo/stereo.cpp:103
    std::string param_base = "params";
    bool xavier = false;
    uint64_t seed = 0;
    int with_xy = 0;
    DevBuf img[2], padded[2], warped, warped_pad, vol, pw, out, labels, out_, out0, qf, p, q, vol3, tvws;
    DevBuf volq;          // BF16 path: the 16-bit fixed-point copy of vol the CRF reads
    bool volq_ok = false; // volq holds the volume of the last compute_volume
    DevBuf gray[2], gtmp, gtmp2, gw, dlist; // census and edge weights
    std::vector<float> dlist_host;          // host copy of the census disparity list
    int filter_size = 7;                    // stereo/stereo_img.cpp:73
    cnncrf_net_t net = nullptr;
    // the net's left features are those of img[0] as it is now (an FP32
    // left-referenced compute_volume since the last image upload): the
    // refinement's re-match keeps them instead of recomputing the same values
    bool left_feats = false;
    cnncrf_slackprop_t solver = nullptr;
    double lb = 0.0;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    bool ev_rec[4] = {false, false, false, false};

    ~cnncrf_stereo()
    {
        destroy_net();
        if (solver) cnncrf_slackprop_destroy(solver);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
    }
    void destroy_net()
    {
        left_feats = false;
        if (net) cnncrf_net_destroy(net);
        net = nullptr;
    }
    bool pairwise() const
    {
        return matching == CNNCRF_MATCH_COLORCNN_PAIRWISE || matching == CNNCRF_MATCH_GRAYCNN_PAIRWISE ||
               matching == CNNCRF_MATCH_CONCATCNN_PAIRWISE;
    }
    int record(int i)
    {
        if (!ev[i]) CNNCRF_CUDA(cudaEventCreate(&ev[i]));
        CNNCRF_CUDA(cudaEventRecord(ev[i], st));
        ev_rec[i] = true;
        return CNNCRF_OK;
    }
    int build_net();
    int compute_volume(int lr);
    int census(int lr);
    int compute_weights(float alpha, float beta, float lambda, int lr);
};

static int log2i(int num) // stereo/stereo.cpp:56-62
{
    int r = 0;
    while (num >>= 1) ++r;
    return r;
}

int cnncrf_stereo::build_net()
{
    if (matching == CNNCRF_MATCH_CENSUS)
        return fail(CNNCRF_EUNSUPPORTED, "CENSUS matching is not on the CNN path and is not built");
    const bool concat = matching == CNNCRF_MATCH_CONCATCNN || matching == CNNCRF_MATCH_CONCATCNN_PAIRWISE;
    bool gray = matching == CNNCRF_MATCH_GRAYCNN || matching == CNNCRF_MATCH_GRAYCNN_PAIRWISE;
    if (!concat && o.topology == CNNCRF_TOPO_REF && num_layers != 3 && num_layers != 5 && num_layers != 7)
        return fail(CNNCRF_EINVAL, "Only {3,5,7} layers are allowed"); // stereo/stereo.cpp:198-202
    cnncrf_net_desc d{};
    d.num_layers = num_layers;
    d.topology = concat ? CNNCRF_TOPO_CONCAT : o.topology; // CONCATCNN: a ConcatStereoNet of num_layers
    d.in_channels = gray ? 1 : (with_xy ? 5 : 3);
    d.feat_channels = concat ? 0 : o.feat_channels;
    d.unary = o.unary;
    d.precision = o.precision;
    d.with_pairwise = pairwise() ? 1 : 0;
    d.pw_channels = o.pw_channels;
    const int pad = net_padding(d);
    CNNCRF_TRY(cnncrf_net_create(&net, &d, 1, H + 2 * pad, W + 2 * pad));
    CNNCRF_TRY(cnncrf_net_set_stream(net, (cnncrf_stream_t)st));
    net->force_interp = false;
    CNNCRF_TRY(cnncrf_net_init(net, dmin, dmax, dstep, 0, vol.as<float>(), pairwise() ? pw.as<float>() : nullptr));
    if (xavier) CNNCRF_TRY(cnncrf_net_init_xavier(net, seed));
    else CNNCRF_TRY(cnncrf_net_set_all_params(net, (param_base + ".npz").c_str())); // stereo/stereo.cpp:188
    size_t pb = sizeof(float) * 4 * (size_t)(W + 2 * pad) * (H + 2 * pad);
    for (int s = 0; s < 2; ++s) CNNCRF_TRY(padded[s].reserve(pb));
    CNNCRF_TRY(warped_pad.reserve(pb));
    return CNNCRF_OK;
}

// calccostvolumecensus on the grey images, lambda 1 (stereo/stereo.cpp:264-268, 290-294)
int cnncrf_stereo::census(int lr)
{
    const size_t n = (size_t)W * H;
    for (int i = 0; i < 2; ++i) CNNCRF_TRY(k::rgb_to_gray(img[i].as<float>(), (long)n, gray[i].as<float>(), st));
    dlist_host.resize((size_t)depth);
    float d = lr ? dmin : -dmax; // disp += disp_step, as the census kernel steps
    for (int z = 0; z < depth; ++z, d += dstep) dlist_host[z] = d;
    CNNCRF_CUDA(cudaMemcpyAsync(dlist.get(), dlist_host.data(), sizeof(float) * depth, cudaMemcpyHostToDevice, st));
    const int a = lr ? 0 : 1;
    return k::census_volume(gray[a].as<float>(), gray[1 - a].as<float>(), W, H, filter_size, dlist.as<float>(), depth,
                            1.0f, vol.as<float>(), st);
}

// computeWeights: calcEdgeImage of the reference side's grey image
// (stereo/stereo.cpp:320-326) into wx, wy
int cnncrf_stereo::compute_weights(float alpha, float beta, float lambda, int lr)
{
    const size_t n = (size_t)W * H;
    CNNCRF_TRY(k::rgb_to_gray(img[lr ? 0 : 1].as<float>(), (long)n, gray[0].as<float>(), st));
    return k::edge_weights(gray[0].as<float>(), W, H, alpha, beta, lambda, gtmp.as<float>(), gtmp2.as<float>(),
                           gw.as<float>(), pw.as<float>(), pw.as<float>() + n, st);
}

int cnncrf_stereo::compute_volume(int lr)
{
    if (!inited) return fail(CNNCRF_ESTATE, "computeVolume before initialize");
    volq_ok = false;
    left_feats = false;
    if (matching == CNNCRF_MATCH_LOAD) return CNNCRF_OK;
    if (matching == CNNCRF_MATCH_CENSUS) return census(lr);
    if (!net) {
        int rc = build_net();
        if (rc != CNNCRF_OK) {
            destroy_net();
            return rc;
        }
    }
    net->force_interp = false;
    float mn = lr ? dmin : -dmax, mx = lr ? dmax : -dmin;
    CNNCRF_TRY(net->set_disparities(mn, mx, dstep, vol.as<float>()));
    if (net->D != depth)
        return fail(CNNCRF_ESHAPE, "Size of provided cost-volume is not correct! disparities do not match! Given size = %d should be %d",
                    depth, net->D);
    int a = lr ? 0 : 1;
    CNNCRF_TRY(k::pad_rgba(img[a].as<float>(), W, H, net->pad, padded[0].as<float>(), st));
    CNNCRF_TRY(k::pad_rgba(img[1 - a].as<float>(), W, H, net->pad, padded[1].as<float>(), st));
    // the BF16 path writes a 16-bit copy of the volume beside it for the CRF
    // (getVolume keeps the FP32 one); the refinement's 3-label predictions
    // (into vol3) do not
    k::UnaryQ16 uq;
    if (o.precision == CNNCRF_BF16 && k::crf_reads_q16(depth) && k::unary_q16(o.unary, &uq)) {
        CNNCRF_TRY(volq.reserve(2 * (size_t)W * H * depth));
        net->volq = volq.get();
        net->vol_fp32 = true;
    }
    const int rc = net->predict(padded[0].as<float>(), padded[1].as<float>());
    volq_ok = rc == CNNCRF_OK && net->volq_valid;
    left_feats = rc == CNNCRF_OK && lr && net->left_ok;
    net->volq = nullptr;
    return rc;
}

extern "C" {

int cnncrf_stereo_default_options(cnncrf_stereo_options *o)
{
    if (!o) return fail(CNNCRF_EINVAL, "null options");
    o->precision = CNNCRF_FP32;
    o->unary = CNNCRF_UNARY_NEG_SOFTMAX;
    o->topology = CNNCRF_TOPO_REF;
    o->feat_channels = 100;
    o->pw_channels = 64;
    o->ref_depth_rounding = 1;
    o->crf_shape = CNNCRF_RHO_STEP;
    o->crf_slack = 0.5f;
    o->huber_eps = 0.1f;
    o->refine_interp = 0;
    return CNNCRF_OK;
}

int cnncrf_stereo_create(cnncrf_stereo_t *s, const cnncrf_stereo_options *opt)
{
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null argument");
    auto *st = new cnncrf_stereo;
    if (opt) st->o = *opt;
    else cnncrf_stereo_default_options(&st->o);
    *s = st;
    return CNNCRF_OK;
}

int cnncrf_stereo_destroy(cnncrf_stereo_t s)
{
    delete s;
    return CNNCRF_OK;
}

int cnncrf_stereo_set_stream(cnncrf_stereo_t s, cnncrf_stream_t stream)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    s->st = (cudaStream_t)stream;
    if (s->net) cnncrf_net_set_stream(s->net, stream);
    if (s->solver) cnncrf_slackprop_set_stream(s->solver, stream);
    return CNNCRF_OK;
}

int cnncrf_stereo_initialize(cnncrf_stereo_t s, int width, int height, float disp_min, float disp_step,
                             float disp_max)
{
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (width < 1 || height < 1) return fail(CNNCRF_EINVAL, "initialize: bad size %dx%d", width, height);
    if (!(disp_step > 0.0f)) return fail(CNNCRF_EINVAL, "initialize: disp_step must be > 0");
    int depth = (int)((disp_max - disp_min) / disp_step + 1); // stereo/stereo.cpp:71
    if (depth < 1) return fail(CNNCRF_EINVAL, "initialize: empty disparity range");
    if (s->o.ref_depth_rounding) depth = std::min(256, 1 << (log2i(depth - 1) + 1)); // :72
    s->W = width, s->H = height, s->depth = depth;
    s->dmin = disp_min, s->dstep = disp_step;
    s->dmax = disp_min + (depth - 1) * disp_step; // :73
    size_t n = (size_t)width * height;
    for (int i = 0; i < 2; ++i) CNNCRF_TRY(s->img[i].reserve(n * 4 * sizeof(float)));
    CNNCRF_TRY(s->warped.reserve(n * 4 * sizeof(float)));
    CNNCRF_TRY(s->vol.reserve(n * depth * sizeof(float)));
    CNNCRF_TRY(s->pw.reserve(2 * n * sizeof(float)));
    CNNCRF_TRY(s->out.reserve(n * sizeof(float)));
    CNNCRF_TRY(s->labels.reserve(n * sizeof(int32_t)));
    CNNCRF_TRY(s->out_.reserve(n * sizeof(float)));
    CNNCRF_TRY(s->out0.reserve(n * sizeof(float)));
    CNNCRF_TRY(s->qf.reserve(2 * n * sizeof(float)));
    CNNCRF_TRY(s->p.reserve(2 * n * sizeof(float)));
    CNNCRF_TRY(s->q.reserve(2 * n * sizeof(float)));
    CNNCRF_TRY(s->tvws.reserve(k::tv_workspace_bytes(width, height)));
    CNNCRF_TRY(s->vol3.reserve(3 * n * sizeof(float)));
    for (int i = 0; i < 2; ++i) CNNCRF_TRY(s->gray[i].reserve(n * sizeof(float)));
    CNNCRF_TRY(s->gtmp.reserve(n * sizeof(float)));
    CNNCRF_TRY(s->gtmp2.reserve(n * sizeof(float)));
    CNNCRF_TRY(s->dlist.reserve(depth * sizeof(float)));
    if (!s->gw.get()) { // the Gaussian of calcEdgeImage never changes
        float w[2 * k::GAUSS_R + 1];
        k::gauss_weights(k::GAUSS_SIGMA, k::GAUSS_R, w);
        CNNCRF_TRY(s->gw.reserve(sizeof w));
        CNNCRF_CUDA(cudaMemcpy(s->gw.get(), w, sizeof w, cudaMemcpyHostToDevice));
    }
    CNNCRF_CUDA(cudaMemsetAsync(s->pw.get(), 0, 2 * n * sizeof(float), s->st));
    s->destroy_net();
    if (s->solver) {
        cnncrf_slackprop_destroy(s->solver);
        s->solver = nullptr;
    }
    s->inited = true;
    return CNNCRF_OK;
}

int cnncrf_stereo_set_matching_function(cnncrf_stereo_t s, int matching)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (matching < 0 || matching > CNNCRF_MATCH_LOAD) return fail(CNNCRF_EINVAL, "unknown matching %d", matching);
    if (matching != s->matching) s->destroy_net();
    s->matching = matching;
    return CNNCRF_OK;
}

int cnncrf_stereo_set_num_layers(cnncrf_stereo_t s, int num_layers)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    s->num_layers = num_layers;
    s->destroy_net(); // stereo/stereo.cpp:354-358
    return CNNCRF_OK;
}

int cnncrf_stereo_set_parameter_file(cnncrf_stereo_t s, const char *base_name)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (base_name) {
        s->param_base = base_name;
        s->xavier = false;
    } else {
        s->xavier = true;
    }
    s->destroy_net(); // stereo/stereo.cpp:360-364
    return CNNCRF_OK;
}

int cnncrf_stereo_set_xavier_seed(cnncrf_stereo_t s, uint64_t seed)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    s->xavier = true;
    s->seed = seed;
    s->destroy_net();
    return CNNCRF_OK;
}

int cnncrf_stereo_set_with_xy(cnncrf_stereo_t s, int with_xy)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (with_xy != s->with_xy) s->destroy_net();
    s->with_xy = with_xy ? 1 : 0;
    return CNNCRF_OK;
}

int cnncrf_stereo_set_color_images(cnncrf_stereo_t s, const float *h_left, const float *h_right)
{
    if (!s || !h_left || !h_right) return fail(CNNCRF_EINVAL, "set_color_images: null argument");
    if (!s->inited) return fail(CNNCRF_ESTATE, "setColorImages before initialize");
    size_t b = sizeof(float) * 4 * (size_t)s->W * s->H;
    s->left_feats = false;
    CNNCRF_CUDA(cudaMemcpyAsync(s->img[0].get(), h_left, b, cudaMemcpyHostToDevice, s->st));
    CNNCRF_CUDA(cudaMemcpyAsync(s->img[1].get(), h_right, b, cudaMemcpyHostToDevice, s->st));
    return CNNCRF_OK;
}

int cnncrf_stereo_set_color_images_device(cnncrf_stereo_t s, const float *d_left, const float *d_right)
{
    if (!s || !d_left || !d_right) return fail(CNNCRF_EINVAL, "set_color_images_device: null argument");
    if (!s->inited) return fail(CNNCRF_ESTATE, "setColorImages before initialize");
    size_t b = sizeof(float) * 4 * (size_t)s->W * s->H;
    s->left_feats = false;
    CNNCRF_CUDA(cudaMemcpyAsync(s->img[0].get(), d_left, b, cudaMemcpyDeviceToDevice, s->st));
    CNNCRF_CUDA(cudaMemcpyAsync(s->img[1].get(), d_right, b, cudaMemcpyDeviceToDevice, s->st));
    return CNNCRF_OK;
}

int cnncrf_stereo_compute_volume(cnncrf_stereo_t s, int lr)
{
    CNNCRF_RANGE("stereo_compute_volume");
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (!s->inited) return fail(CNNCRF_ESTATE, "computeVolume before initialize");
    CNNCRF_TRY(s->record(0));
    CNNCRF_TRY(s->compute_volume(lr));
    return s->record(1);
}

int cnncrf_stereo_compute_slack_propagation(cnncrf_stereo_t s, float C1, float C2, float delta, int iterations,
                                            float alpha, float beta, float lambda_reg, int lr)
{
    CNNCRF_RANGE("stereo_compute_slack_propagation");
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (!s->inited) return fail(CNNCRF_ESTATE, "computeSlackPropagation before initialize");
    CNNCRF_TRY(s->record(0));
    CNNCRF_TRY(s->compute_volume(lr));
    CNNCRF_TRY(s->record(1));
    size_t n = (size_t)s->W * s->H;
    if (s->pairwise()) // the pairwise CNN's weights, times lambda (stereo/stereo.cpp:136-137)
        CNNCRF_TRY(k::scale(s->pw.as<float>(), (long)(2 * n), lambda_reg, s->st));
    else // image-gradient edge weights (stereo/stereo.cpp:132-133)
        CNNCRF_TRY(s->compute_weights(alpha, beta, lambda_reg, lr));
    if (!s->solver) {
        CNNCRF_TRY(cnncrf_slackprop_create(&s->solver));
        CNNCRF_TRY(cnncrf_slackprop_init(s->solver, s->vol.as<float>(), s->W, s->H, s->depth, s->labels.as<int32_t>()));
    }
    cnncrf_slackprop_set_stream(s->solver, (cnncrf_stream_t)s->st);
    k::UnaryQ16 uq{1.0f, 0.0f};
    k::unary_q16(s->o.unary, &uq);
    k::slackprop_set_costq(s->solver, s->volq_ok ? s->volq.get() : nullptr, uq);
    CNNCRF_TRY(cnncrf_slackprop_set_op(s->solver, "L1", C1));
    CNNCRF_TRY(cnncrf_slackprop_set_op(s->solver, "L2", C2));
    CNNCRF_TRY(cnncrf_slackprop_set_op(s->solver, "delta", delta));
    CNNCRF_TRY(cnncrf_slackprop_set_op(s->solver, "total_it", iterations));
    CNNCRF_TRY(cnncrf_slackprop_set_op(s->solver, "shape", s->o.crf_shape));
    CNNCRF_TRY(cnncrf_slackprop_set_op(s->solver, "slack", s->o.crf_slack));
    CNNCRF_TRY(cnncrf_slackprop_update_w(s->solver, s->pw.as<float>(), s->pw.as<float>() + n));
    CNNCRF_TRY(cnncrf_slackprop_execute(s->solver));
    CNNCRF_TRY(cnncrf_slackprop_lower_bound(s->solver, &s->lb));
    if (lr) CNNCRF_TRY(k::remap(s->out.as<float>(), s->labels.as<int32_t>(), (long)n, s->dmin, s->dstep, s->st));
    else CNNCRF_TRY(k::remap(s->out.as<float>(), s->labels.as<int32_t>(), (long)n, -s->dmax, s->dstep, s->st));
    return s->record(2);
}

int cnncrf_stereo_set_filter_size(cnncrf_stereo_t s, int filter_size)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (filter_size < 1 || filter_size > 16) return fail(CNNCRF_EINVAL, "filter size %d outside 1..16", filter_size);
    s->filter_size = filter_size;
    return CNNCRF_OK;
}

int cnncrf_stereo_compute_weights(cnncrf_stereo_t s, float alpha, float beta, float lambda_reg, int lr)
{
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (!s->inited) return fail(CNNCRF_ESTATE, "computeWeights before initialize");
    return s->compute_weights(alpha, beta, lambda_reg, lr);
}

int cnncrf_stereo_fuse_quad_fit_direct(cnncrf_stereo_t s)
{
    CNNCRF_RANGE("stereo_fuse_quad_fit_direct");
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (!s->solver) return fail(CNNCRF_ESTATE, "fuseQuadFitDirect needs a computeSlackPropagation first");
    float *c1 = nullptr;
    CNNCRF_TRY(cnncrf_slackprop_get_c1(s->solver, &c1)); // solver->get_C1() (stereo/stereo.cpp:408)
    return k::quadfit_direct(s->out.as<float>(), c1, (long)s->W * s->H, s->depth, s->dmin, s->dstep, s->st);
}

int cnncrf_stereo_compute_argmax(cnncrf_stereo_t s, int lr)
{
    CNNCRF_RANGE("stereo_compute_argmax");
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (!s->inited) return fail(CNNCRF_ESTATE, "computeArgMax before initialize");
    CNNCRF_TRY(s->record(0));
    CNNCRF_TRY(s->compute_volume(lr));
    CNNCRF_TRY(s->record(1));
    size_t n = (size_t)s->W * s->H;
    CNNCRF_TRY(k::argmin(s->out.as<float>(), s->vol.as<float>(), (long)n, s->depth, lr ? s->dmin : -s->dmax,
                         s->dstep, s->st));
    return s->record(2);
}

int cnncrf_stereo_fuse_thuber_quad_fit(cnncrf_stereo_t s, float lambda_reg, float C, int iterations, int warps)
{
    CNNCRF_RANGE("stereo_fuse_thuber_quad_fit");
    clear_error();
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    if (!s->net || !s->pairwise())
        return fail(CNNCRF_ESTATE, "fuseTHuberQuadFit needs a COLORPAIR net that has computed a volume");
    cnncrf_net *net = s->net;
    cudaStream_t st = s->st;
    int W = s->W, H = s->H;
    size_t n = (size_t)W * H;
    float lam_c = 1.0f / lambda_reg; // stereo/stereo.cpp:395
    float step = s->dstep;
    float hq = (float)((double)step * 0.25), mn = (float)(-(double)step * 0.25);
    CNNCRF_TRY(k::pad_rgba(s->img[0].as<float>(), W, H, net->pad, s->padded[0].as<float>(), st));
    for (int w = 0; w < warps; ++w) {
        CNNCRF_TRY(k::warp_rgba(s->warped.as<float>(), s->img[1].as<float>(), s->out.as<float>(), W, H, st));
        CNNCRF_TRY(k::pad_rgba(s->warped.as<float>(), W, H, net->pad, s->warped_pad.as<float>(), st));
        net->force_interp = s->o.refine_interp != 0;
        CNNCRF_TRY(net->set_disparities(mn, hq, hq, s->vol3.as<float>()));
        if (net->D != 3) return fail(CNNCRF_ESHAPE, "refinement volume has %d labels, expected 3", net->D);
        // the left input is padded[0] of img[0] as in the matching: its features stay valid
        net->reuse_left = s->left_feats;
        const int rc = net->predict(s->padded[0].as<float>(), s->warped_pad.as<float>());
        s->left_feats = rc == CNNCRF_OK && net->left_ok;
        CNNCRF_TRY(rc);
        net->force_interp = false;
        CNNCRF_TRY(k::tv_fit(s->vol3.as<float>(), s->qf.as<float>(), W, H, step, lam_c, st));
        CNNCRF_CUDA(cudaMemcpyAsync(s->out0.get(), s->out.get(), n * sizeof(float), cudaMemcpyDeviceToDevice, st));
        // predict rewrote wx / wy (they alias the pairwise output) without lambda
        // p = q = 0 before the first warp (stereo/stereo.cu:1133-1135); later warps continue from them
        CNNCRF_TRY(k::tv_iterate(s->out.as<float>(), s->out_.as<float>(), s->out0.as<float>(), s->qf.as<float>(),
                                 s->p.as<float>(), s->q.as<float>(), s->pw.as<float>(), s->pw.as<float>() + n, W, H, C,
                                 s->o.huber_eps, step, iterations, s->tvws.get(), s->tvws.size(), w == 0, st));
    }
    return s->record(3);
}

int cnncrf_stereo_get_output(cnncrf_stereo_t s, float *h_out)
{
    if (!s || !h_out) return fail(CNNCRF_EINVAL, "null argument");
    CNNCRF_CUDA(cudaMemcpyAsync(h_out, s->out.get(), sizeof(float) * (size_t)s->W * s->H, cudaMemcpyDeviceToHost, s->st));
    CNNCRF_CUDA(cudaStreamSynchronize(s->st));
    return CNNCRF_OK;
}

int cnncrf_stereo_get_output_device(cnncrf_stereo_t s, const float **d_out)
{
    if (!s || !d_out) return fail(CNNCRF_EINVAL, "null argument");
    *d_out = s->out.as<float>();
    return CNNCRF_OK;
}

int cnncrf_stereo_get_labels_device(cnncrf_stereo_t s, const int32_t **d_labels)
{
    if (!s || !d_labels) return fail(CNNCRF_EINVAL, "null argument");
    *d_labels = s->labels.as<int32_t>();
    return CNNCRF_OK;
}

int cnncrf_stereo_get_volume_device(cnncrf_stereo_t s, const float **d_volume)
{
    if (!s || !d_volume) return fail(CNNCRF_EINVAL, "null argument");
    *d_volume = s->vol.as<float>();
    return CNNCRF_OK;
}

int cnncrf_stereo_get_weights_device(cnncrf_stereo_t s, const float **d_wx, const float **d_wy)
{
    if (!s || !d_wx || !d_wy) return fail(CNNCRF_EINVAL, "null argument");
    *d_wx = s->pw.as<float>();
    *d_wy = s->pw.as<float>() + (size_t)s->W * s->H;
    return CNNCRF_OK;
}

int cnncrf_stereo_get_depth(cnncrf_stereo_t s, int *depth)
{
    if (!s || !depth) return fail(CNNCRF_EINVAL, "null argument");
    *depth = s->depth;
    return CNNCRF_OK;
}

int cnncrf_stereo_lower_bound(cnncrf_stereo_t s, double *lb)
{
    if (!s || !lb) return fail(CNNCRF_EINVAL, "null argument");
    *lb = s->lb;
    return CNNCRF_OK;
}

int cnncrf_stereo_stage_times(cnncrf_stereo_t s, float *cnn_ms, float *corr_ms, float *crf_ms, float *refine_ms)
{
    if (!s) return fail(CNNCRF_EINVAL, "null stereo");
    CNNCRF_CUDA(cudaStreamSynchronize(s->st));
    float t01 = 0, t12 = 0, t23 = 0;
    if (s->ev_rec[0] && s->ev_rec[1]) CNNCRF_CUDA(cudaEventElapsedTime(&t01, s->ev[0], s->ev[1]));
    if (s->ev_rec[1] && s->ev_rec[2]) CNNCRF_CUDA(cudaEventElapsedTime(&t12, s->ev[1], s->ev[2]));
    if (s->ev_rec[2] && s->ev_rec[3]) CNNCRF_CUDA(cudaEventElapsedTime(&t23, s->ev[2], s->ev[3]));
    if (cnn_ms) *cnn_ms = t01;
    if (corr_ms) *corr_ms = 0.0f; // fused into the CNN stage
    if (crf_ms) *crf_ms = t12;
    if (refine_ms) *refine_ms = t23;
    return CNNCRF_OK;
}

} // extern "C"
