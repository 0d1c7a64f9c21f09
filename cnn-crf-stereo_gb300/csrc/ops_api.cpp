// ops_api.cpp -- C ABI of the standalone operators: correlation, the CRF
// solver (function and slack_prop_2D_alg-style object), remap and the TV
// refinement kernels.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "common.h"
#include "kernels.h"

using namespace cnncrf;

struct cnncrf_slackprop {
    cudaStream_t st = nullptr;
    const float *cost = nullptr;
    const void *costq = nullptr; // a 16-bit fixed-point copy of cost the solve reads instead (BF16 Stereo path)
    k::UnaryQ16 q{1.0f, 0.0f};
    int W = 0, H = 0, D = 0;
    int32_t *labels = nullptr;
    const float *wx = nullptr, *wy = nullptr;
    cnncrf_crf_options ops{};
    DevBuf ws, c1;
    double lb = 0.0;
    bool ran = false;
};

int cnncrf::k::crf_params(const cnncrf_crf_options *opt, k::CrfParams *p)
{
    int delta = (int)opt->delta;
    if ((float)delta != opt->delta || delta < 1 || delta > 4)
        return fail(CNNCRF_EUNSUPPORTED, "crf: delta %g must be an integer in 1..4", opt->delta);
    if (opt->shape != CNNCRF_RHO_STEP && opt->shape != CNNCRF_RHO_LINEAR)
        return fail(CNNCRF_EINVAL, "crf: shape %d", opt->shape);
    p->L1 = opt->L1;
    p->L2 = opt->L2;
    p->delta = delta;
    p->shape = opt->shape;
    p->slack = opt->slack;
    return CNNCRF_OK;
}

// The BF16 Stereo path hands the solver the 16-bit copy of its volume that the
// correlation wrote (null: the FP32 volume); not part of the C ABI.
void cnncrf::k::slackprop_set_costq(cnncrf_slackprop *sp, const void *costq, UnaryQ16 q)
{
    if (sp) sp->costq = costq, sp->q = q;
}

extern "C" {

int cnncrf_set_conv_pairs(int enable)
{
    k::conv_tc_set_pairs(enable != 0);
    return CNNCRF_OK;
}

int cnncrf_get_conv_pairs(int *enable)
{
    if (!enable) return fail(CNNCRF_EINVAL, "null argument");
    *enable = k::conv_tc_pairs() ? 1 : 0;
    return CNNCRF_OK;
}

// StereoCorrelation::forward static entry (stereo/operators/stereocorrelation.cpp:146-152)
int cnncrf_correlation_forward(const float *d_input0, const float *d_input1, const float *h_disparities,
                               float *d_output, int n, int c, int h, int w, int num_disps,
                               cnncrf_stream_t stream)
{
    clear_error();
    if (!d_input0 || !d_input1 || !h_disparities || !d_output) return fail(CNNCRF_EINVAL, "correlation: null");
    if (n != 1) return fail(CNNCRF_EUNSUPPORTED, "correlation: only n = 1");
    if (c < 1 || h < 1 || w < 1 || num_disps < 1) return fail(CNNCRF_EINVAL, "correlation: bad size");
    cudaStream_t st = (cudaStream_t)stream;
    // NCHW inputs -> NHWC staging (the kernel reads pixel-contiguous features)
    DevBuf l, r, dl;
    size_t np = (size_t)h * w;
    CNNCRF_TRY(l.reserve(np * c * sizeof(float)));
    CNNCRF_TRY(r.reserve(np * c * sizeof(float)));
    CNNCRF_TRY(dl.reserve(sizeof(float) * num_disps));
    CNNCRF_TRY(k::nchw_to_nhwc(d_input0, l.as<float>(), c, (long)np, st));
    CNNCRF_TRY(k::nchw_to_nhwc(d_input1, r.as<float>(), c, (long)np, st));
    CNNCRF_CUDA(cudaMemcpyAsync(dl.get(), h_disparities, sizeof(float) * num_disps, cudaMemcpyHostToDevice, st));
    float v = num_disps >= 2 ? h_disparities[1] : h_disparities[0];
    bool interp = std::fabs(v - std::round(v)) > 0.001f;
    int omin = 1 << 30, omax = -(1 << 30);
    for (int i = 0; i < num_disps; ++i) {
        float s = h_disparities[i];
        int a = interp ? (int)std::floor(s) - 1 : (int)s, b = interp ? (int)std::floor(s) + 2 : (int)s;
        omin = std::min(omin, a), omax = std::max(omax, b);
    }
    CNNCRF_TRY(k::correlation(l.as<float>(), r.as<float>(), h, w, c, dl.as<float>(), num_disps, omin, omax, interp,
                              -1, d_output, st));
    CNNCRF_CUDA(cudaStreamSynchronize(st));
    return CNNCRF_OK;
}

int cnncrf_crf_default_options(cnncrf_crf_options *o)
{
    if (!o) return fail(CNNCRF_EINVAL, "null options");
    o->L1 = 1.0f;
    o->L2 = 12.0f;
    o->delta = 2.0f;
    o->total_it = 4;
    o->shape = CNNCRF_RHO_STEP;
    o->slack = 0.5f;
    return CNNCRF_OK;
}

int cnncrf_crf_workspace_size(int width, int height, int depth, size_t *bytes)
{
    if (!bytes || width < 1 || height < 1 || depth < 1) return fail(CNNCRF_EINVAL, "workspace_size: bad argument");
    *bytes = k::crf_workspace_bytes(width, height, depth);
    return CNNCRF_OK;
}


int cnncrf_conv_tuning_count(int *n)
{
    if (!n) return fail(CNNCRF_EINVAL, "null argument");
    *n = k::conv_forms_count();
    return CNNCRF_OK;
}

int cnncrf_conv_tuning_get(int index, int shape[10], int *pair, int *stages, float *ms)
{
    if (!shape || !pair || !stages || !ms) return fail(CNNCRF_EINVAL, "null argument");
    k::ConvForm f;
    if (!k::conv_form_entry(index, shape, &f, ms)) return fail(CNNCRF_EINVAL, "conv tuning: no entry %d", index);
    *pair = f.pair, *stages = f.stages;
    return CNNCRF_OK;
}

int cnncrf_conv_tuning_clear(void)
{
    k::conv_forms_clear();
    return CNNCRF_OK;
}

int cnncrf_selftest_bounded_wait(int polls, int arrive, cnncrf_stream_t stream)
{
    clear_error();
    return k::selftest_bounded_wait(polls, arrive, (cudaStream_t)stream);
}

int cnncrf_crf_solve(const float *d_cost, const float *d_wx, const float *d_wy, int width, int height, int depth,
                     const cnncrf_crf_options *opt, int32_t *d_labels, double *lower_bound, void *d_workspace,
                     size_t workspace_bytes, cnncrf_stream_t stream)
{
    CNNCRF_RANGE("crf_solve");
    clear_error();
    if (!opt) return fail(CNNCRF_EINVAL, "crf: null options");
    k::CrfParams p;
    CNNCRF_TRY(k::crf_params(opt, &p));
    return k::crf_solve(d_cost, d_wx, d_wy, width, height, depth, p, opt->total_it, d_labels, d_workspace,
                        workspace_bytes, lower_bound, (cudaStream_t)stream);
}

int cnncrf_crf_autotune(const float *d_cost, const float *d_wx, const float *d_wy, int width, int height, int depth,
                        const cnncrf_crf_options *opt, void *d_workspace, size_t workspace_bytes,
                        cnncrf_stream_t stream)
{
    clear_error();
    if (!opt) return fail(CNNCRF_EINVAL, "crf: null options");
    k::CrfParams p;
    CNNCRF_TRY(k::crf_params(opt, &p));
    return k::crf_autotune(d_cost, d_wx, d_wy, 0, width, height, depth, 1, p, d_workspace, workspace_bytes,
                           (cudaStream_t)stream);
}

int cnncrf_slackprop_create(cnncrf_slackprop_t *sp)
{
    if (!sp) return fail(CNNCRF_EINVAL, "null argument");
    *sp = new cnncrf_slackprop;
    cnncrf_crf_default_options(&(*sp)->ops);
    return CNNCRF_OK;
}

int cnncrf_slackprop_destroy(cnncrf_slackprop_t sp)
{
    delete sp;
    return CNNCRF_OK;
}

int cnncrf_slackprop_set_stream(cnncrf_slackprop_t sp, cnncrf_stream_t stream)
{
    if (!sp) return fail(CNNCRF_EINVAL, "null solver");
    sp->st = (cudaStream_t)stream;
    return CNNCRF_OK;
}

int cnncrf_slackprop_init(cnncrf_slackprop_t sp, const float *d_cost, int width, int height, int depth,
                          int32_t *d_labels)
{
    clear_error();
    if (!sp || !d_cost || !d_labels) return fail(CNNCRF_EINVAL, "slackprop init: null argument");
    if (width < 1 || height < 1 || depth < 1 || depth > 256)
        return fail(CNNCRF_EINVAL, "slackprop init: bad size %dx%dx%d", width, height, depth);
    sp->cost = d_cost, sp->W = width, sp->H = height, sp->D = depth, sp->labels = d_labels;
    CNNCRF_TRY(sp->ws.reserve(k::crf_workspace_bytes(width, height, depth)));
    sp->ran = false;
    return CNNCRF_OK;
}

int cnncrf_slackprop_set_op(cnncrf_slackprop_t sp, const char *name, double value)
{
    if (!sp || !name) return fail(CNNCRF_EINVAL, "null argument");
    std::string n(name);
    if (n == "L1") sp->ops.L1 = (float)value;
    else if (n == "L2") sp->ops.L2 = (float)value;
    else if (n == "delta") sp->ops.delta = (float)value;
    else if (n == "total_it") sp->ops.total_it = (int)value;
    else if (n == "slack") sp->ops.slack = (float)value;
    else if (n == "shape") sp->ops.shape = (int)value;
    else return fail(CNNCRF_EINVAL, "slackprop: unknown option '%s'", name);
    return CNNCRF_OK;
}

int cnncrf_slackprop_update_w(cnncrf_slackprop_t sp, const float *d_wx, const float *d_wy)
{
    if (!sp || !d_wx || !d_wy) return fail(CNNCRF_EINVAL, "null argument");
    sp->wx = d_wx, sp->wy = d_wy;
    return CNNCRF_OK;
}

int cnncrf_slackprop_execute(cnncrf_slackprop_t sp)
{
    clear_error();
    if (!sp || !sp->cost) return fail(CNNCRF_ESTATE, "slackprop: execute before init");
    if (!sp->wx) return fail(CNNCRF_ESTATE, "slackprop: execute before update_W");
    k::CrfParams p;
    CNNCRF_TRY(k::crf_params(&sp->ops, &p));
    CNNCRF_TRY(k::crf_solve(sp->cost, sp->wx, sp->wy, sp->W, sp->H, sp->D, p, sp->ops.total_it, sp->labels,
                            sp->ws.get(), sp->ws.size(), &sp->lb, sp->st, sp->costq, sp->q));
    sp->ran = true;
    return CNNCRF_OK;
}

int cnncrf_slackprop_lower_bound(cnncrf_slackprop_t sp, double *lb)
{
    if (!sp || !lb) return fail(CNNCRF_EINVAL, "null argument");
    if (!sp->ran) return fail(CNNCRF_ESTATE, "slackprop: LB before execute");
    *lb = sp->lb;
    return CNNCRF_OK;
}

int cnncrf_slackprop_get_c1(cnncrf_slackprop_t sp, float **d_c1)
{
    if (!sp || !d_c1) return fail(CNNCRF_EINVAL, "null argument");
    if (!sp->ran || sp->ops.total_it <= 0) return fail(CNNCRF_ESTATE, "slackprop: get_C1 before execute");
    long n = (long)sp->W * sp->H * sp->D;
    CNNCRF_TRY(sp->c1.reserve(sizeof(float) * n));
    CNNCRF_TRY(k::crf_c1(sp->cost, sp->ws.get(), n, sp->c1.as<float>(), sp->st, sp->D, sp->costq, sp->q));
    *d_c1 = sp->c1.as<float>();
    return CNNCRF_OK;
}

int cnncrf_remap_solution(float *d_out, const int32_t *d_labels, int width, int height, float disp_min,
                          float disp_step, cnncrf_stream_t stream)
{
    if (!d_out || !d_labels) return fail(CNNCRF_EINVAL, "remap: null argument");
    return k::remap(d_out, d_labels, (long)width * height, disp_min, disp_step, (cudaStream_t)stream);
}

int cnncrf_warp_image(float *d_out_rgba, const float *d_in_rgba, const float *d_u, int width, int height,
                      cnncrf_stream_t stream)
{
    if (!d_out_rgba || !d_in_rgba || !d_u) return fail(CNNCRF_EINVAL, "warp: null argument");
    return k::warp_rgba(d_out_rgba, d_in_rgba, d_u, width, height, (cudaStream_t)stream);
}

int cnncrf_tv_fit(const float *d_volume3, float *d_qf, int width, int height, float disp_step, float lambda_census,
                  cnncrf_stream_t stream)
{
    if (!d_volume3 || !d_qf) return fail(CNNCRF_EINVAL, "tv_fit: null argument");
    return k::tv_fit(d_volume3, d_qf, width, height, disp_step, lambda_census, (cudaStream_t)stream);
}

int cnncrf_tv_workspace_size(int width, int height, size_t *bytes)
{
    if (!bytes || width < 1 || height < 1) return fail(CNNCRF_EINVAL, "tv_workspace_size: bad argument");
    *bytes = k::tv_workspace_bytes(width, height);
    return CNNCRF_OK;
}

int cnncrf_tv_iterate(float *d_u, float *d_u_, const float *d_u0, const float *d_qf, float *d_p, float *d_q,
                      const float *d_wx, const float *d_wy, int width, int height, float C, float huber_eps,
                      float disp_step, int iterations, void *d_workspace, size_t workspace_bytes,
                      cnncrf_stream_t stream)
{
    clear_error();
    if (!d_u || !d_u_ || !d_u0 || !d_qf || !d_p || !d_q || !d_wx || !d_wy)
        return fail(CNNCRF_EINVAL, "tv_iterate: null argument");
    // p = q = 0 at the start (stereo/stereo.cu:1133-1135)
    return k::tv_iterate(d_u, d_u_, d_u0, d_qf, d_p, d_q, d_wx, d_wy, width, height, C, huber_eps, disp_step,
                         iterations, d_workspace, workspace_bytes, true, (cudaStream_t)stream);
}

// ---------------------------------------------------------------- census, edge weights, QuadDirect, LR check

int cnncrf_rgb_to_gray(const float *d_rgba, float *d_gray, int width, int height, cnncrf_stream_t stream)
{
    clear_error();
    if (!d_rgba || !d_gray || width < 1 || height < 1) return fail(CNNCRF_EINVAL, "rgb_to_gray: bad argument");
    return k::rgb_to_gray(d_rgba, (long)width * height, d_gray, (cudaStream_t)stream);
}

int cnncrf_census_volume(const float *d_gray_ref, const float *d_gray_other, int width, int height, int filter_size,
                         float disp_min, float disp_step, int depth, float lambda, float *d_volume,
                         cnncrf_stream_t stream)
{
    clear_error();
    if (!d_gray_ref || !d_gray_other || !d_volume || width < 1 || height < 1 || depth < 1)
        return fail(CNNCRF_EINVAL, "census_volume: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<float> l((size_t)depth);
    float d = disp_min;
    for (int z = 0; z < depth; ++z, d += disp_step) l[z] = d;
    DevBuf dl;
    CNNCRF_TRY(dl.reserve(sizeof(float) * depth));
    CNNCRF_CUDA(cudaMemcpyAsync(dl.get(), l.data(), sizeof(float) * depth, cudaMemcpyHostToDevice, st));
    CNNCRF_TRY(k::census_volume(d_gray_ref, d_gray_other, width, height, filter_size, dl.as<float>(), depth, lambda,
                                d_volume, st));
    CNNCRF_CUDA(cudaStreamSynchronize(st)); // the list buffer is freed on return
    return CNNCRF_OK;
}

int cnncrf_edge_weights(const float *d_gray, int width, int height, float alpha, float beta, float lambda,
                        float *d_wx, float *d_wy, cnncrf_stream_t stream)
{
    clear_error();
    if (!d_gray || !d_wx || !d_wy || width < 1 || height < 1) return fail(CNNCRF_EINVAL, "edge_weights: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)width * height;
    float w[2 * k::GAUSS_R + 1];
    k::gauss_weights(k::GAUSS_SIGMA, k::GAUSS_R, w);
    DevBuf t1, t2, gw;
    CNNCRF_TRY(t1.reserve(n * sizeof(float)));
    CNNCRF_TRY(t2.reserve(n * sizeof(float)));
    CNNCRF_TRY(gw.reserve(sizeof w));
    CNNCRF_CUDA(cudaMemcpyAsync(gw.get(), w, sizeof w, cudaMemcpyHostToDevice, st));
    CNNCRF_TRY(k::edge_weights(d_gray, width, height, alpha, beta, lambda, t1.as<float>(), t2.as<float>(),
                               gw.as<float>(), d_wx, d_wy, st));
    CNNCRF_CUDA(cudaStreamSynchronize(st)); // the scratch buffers are freed on return
    return CNNCRF_OK;
}

int cnncrf_quad_fit_direct(float *d_u, const float *d_c1, int width, int height, int depth, float disp_min,
                           float disp_step, cnncrf_stream_t stream)
{
    clear_error();
    if (!d_u || !d_c1 || width < 1 || height < 1 || depth < 1 || !(disp_step > 0.0f))
        return fail(CNNCRF_EINVAL, "quad_fit_direct: bad argument");
    return k::quadfit_direct(d_u, d_c1, (long)width * height, depth, disp_min, disp_step, (cudaStream_t)stream);
}

int cnncrf_left_right_check(const float *d_left, const float *d_right, int width, int height, float threshold,
                            float *d_out, cnncrf_stream_t stream)
{
    clear_error();
    if (!d_left || !d_right || !d_out || width < 1 || height < 1)
        return fail(CNNCRF_EINVAL, "left_right_check: bad argument");
    return k::lr_check(d_left, d_right, width, height, threshold, d_out, (cudaStream_t)stream);
}

} // extern "C"
