/*
 * cnncrf.h -- C ABI of the GB300-native CNN-CRF stereo hot path (libcnncrf.so).
 *
 * Every entry point replaces one call of the reference's C++ API for the path
 * (VLOGroup/cnn-crf-stereo); the citation above each declaration names it.
 * Plain pointers, sizes and a cudaStream_t only: no C++ or torch types.
 *
 * Conventions
 *  - Every function returns a cnncrf_status; the reference aborted with
 *    exit(-1) (stereo/error_util.h:29-52), this library never aborts.  The
 *    message of the last failure on the calling thread is cnncrf_last_error().
 *  - "d_" pointers are device pointers, "h_" pointers are host pointers.
 *  - Images are RGBA float (4 interleaved channels), rows packed (pitch =
 *    4*width floats) -- the iu::ImageGpu_32f_C4 the reference passes around.
 *  - Cost volumes are H x W x D floats, D fastest ("NHWC" with C = D), the
 *    layout of stereo/stereo.cpp:82,219-220 and slack_prop {K,W,H}.
 *  - Pairwise weights are [2][H][W] floats, channel 0 = wx (edge (y,x)-(y,x+1)),
 *    channel 1 = wy (edge (y,x)-(y+1,x)), aliasing as in stereo/stereo.cpp:84-86.
 *  - Handles are not shared between threads; use one handle per host thread.
 *    Nothing is process-global except the error message (thread-local).
 *  - All work is enqueued on the stream given to the handle (default: the
 *    legacy default stream); functions that return host data synchronise it.
 */
#ifndef CNNCRF_H
#define CNNCRF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CNNCRF_ABI_VERSION 1

typedef struct CUstream_st *cnncrf_stream_t; /* == cudaStream_t */

typedef enum cnncrf_status {
    CNNCRF_OK = 0,
    CNNCRF_EINVAL = 1,      /* bad argument (null pointer, negative size, ...) */
    CNNCRF_ESHAPE = 2,      /* tensor / npz array shape mismatch */
    CNNCRF_ENOMEM = 3,      /* device or host allocation failed */
    CNNCRF_ECUDA = 4,       /* CUDA runtime / driver error */
    CNNCRF_ETIMEOUT = 5,    /* a bounded device wait ran out (kernel error flag) */
    CNNCRF_EIO = 6,         /* file missing / unreadable / corrupt */
    CNNCRF_ESTATE = 7,      /* call order violated (e.g. predict before init) */
    CNNCRF_EUNSUPPORTED = 8 /* valid in the reference, not built here */
} cnncrf_status;

/* Matching functions; values equal the reference enum (stereo/stereo.h:29-38). */
typedef enum cnncrf_matching {
    CNNCRF_MATCH_COLORCNN = 0,
    CNNCRF_MATCH_GRAYCNN = 1,
    CNNCRF_MATCH_CONCATCNN = 2,          /* ConcatStereoNet (CNNCRF_TOPO_CONCAT), FP32 */
    CNNCRF_MATCH_GRAYCNN_PAIRWISE = 3,
    CNNCRF_MATCH_COLORCNN_PAIRWISE = 4,  /* "COLORPAIR" on the command line */
    CNNCRF_MATCH_CONCATCNN_PAIRWISE = 5, /* the same with its pairwise weights */
    CNNCRF_MATCH_CENSUS = 6,             /* census cost + image-gradient edge weights */
    CNNCRF_MATCH_LOAD = 7                /* volume supplied by the caller */
} cnncrf_matching;

typedef enum cnncrf_precision {
    CNNCRF_FP32 = 0, /* SIMT FP32, bit-exact against the CPU oracle */
    CNNCRF_BF16 = 1  /* tcgen05 BF16 operands, FP32 accumulation */
} cnncrf_precision;

typedef enum cnncrf_unary {
    CNNCRF_UNARY_NEG_SOFTMAX = 0, /* -softmax_d(<fL,fR>) (stereo/stereonet.cpp:136-139,309,318) */
    CNNCRF_UNARY_ONE_MINUS_DOT = 1 /* 1 - <fL,fR> on L2-normalised features */
} cnncrf_unary;

typedef enum cnncrf_topology {
    CNNCRF_TOPO_REF = 0,    /* 3x3 first layer, 2x2 layers after (stereo/stereonet.cpp:69-133) */
    CNNCRF_TOPO_ALL3X3 = 1, /* every layer 3x3 */
    /* ConcatStereoNet (stereo/concatstereonet.cpp:28-127), FP32 only: num_layers
       one of 3, 5, 7, 10, 15, 20, 25, 33, 50, 100, with the growth rate g the
       reference's constructor gives that depth (33, 20, 14, 10, 7, 5, 4, 3, 2,
       1).  Every layer is a 3x3 conv with zero padding 1 to g channels, bias and
       tanh, fed the previous layer's output; the features are all layers'
       outputs side by side, g * num_layers channels (feat_channels must be 0 or
       that number).  No mirror padding (cnncrf_net_padding 0,
       stereo/stereo.cpp:214-216).  The pairwise weights: one 3x3 conv of the
       features to 2 channels, zero padding 1, no bias, |tanh|.  The reference
       declares this net but never runs it (stereo/stereo.cpp:237-254 builds
       only ColorStereoNet; its correlation is declared on the input's channels
       and its pairwise conv on 100), so these are this library's readings:
       the correlation over the concatenated features, the pairwise conv over
       them, and |.| to keep the CRF's weights non-negative. */
    CNNCRF_TOPO_CONCAT = 2
} cnncrf_topology;

typedef enum cnncrf_pairwise_shape {
    CNNCRF_RHO_STEP = 0,  /* rho(0)=0, rho(t)=L1 for 1<=|t|<=delta, L2 beyond */
    CNNCRF_RHO_LINEAR = 1 /* rho(t)=min(L1*|t|, L2) for |t|<=delta, L2 beyond */
} cnncrf_pairwise_shape;

/* ---------------------------------------------------------------- errors */

/* Message of the last failed call on this thread ("" if none). */
const char *cnncrf_last_error(void);
/* Library ABI version (CNNCRF_ABI_VERSION). */
int cnncrf_abi_version(void);

/* The BF16 path's tensor-core convolutions (layers 2..L, the pairwise net's
   second layer, a training step's input gradients) as 2-CTA pairs whose MMAs
   span both SMs (tcgen05 cta_group::2): on by default where the device
   co-schedules the clusters.  0 runs them on single CTAs.  Process-wide.  The
   two forms differ at most in FP32 summation order.  No reference
   counterpart (a GB300 execution choice). */
int cnncrf_set_conv_pairs(int enable);
int cnncrf_get_conv_pairs(int *enable);
/* The tensor-core convolutions' tuned launch forms (no reference
 * counterpart).  cnncrf_batch_autotune times every form of each of its nets'
 * convolutions -- 2-CTA pairs or single CTAs, 2 to 4 pipeline stages -- and
 * enters the fastest per layer shape in a process-wide table that later
 * launches of that shape use (every form gives the same bits).
 * shape = n_img, Hin, Win, cp_in, cin, np, cout, kh, kw, mode. */
int cnncrf_conv_tuning_count(int *n);
int cnncrf_conv_tuning_get(int index, int shape[10], int *pair, int *stages, float *ms);
int cnncrf_conv_tuning_clear(void);

/* ---------------------------------------------------------------- StereoNet */

typedef struct cnncrf_net *cnncrf_net_t;

typedef struct cnncrf_net_desc {
    int num_layers;    /* feature CNN depth (REF topology: 3, 5 or 7) */
    int topology;      /* cnncrf_topology */
    int in_channels;   /* 1 (gray), 3 (RGB) or 5 (RGB + normalised x,y) */
    int feat_channels; /* 100 in the reference */
    int unary;         /* cnncrf_unary */
    int precision;     /* cnncrf_precision */
    int with_pairwise; /* build the pairwise-weight CNN (COLORPAIR) */
    int pw_channels;   /* 64 in the reference */
} cnncrf_net_desc;

/* StereoNet(numLayers, n, c, h, w) (stereo/stereonet.h:30) / ColorStereoNet
 * (stereo/colorstereonet.h:25).  h, w are the PADDED input size.  Only n = 1. */
int cnncrf_net_create(cnncrf_net_t *net, const cnncrf_net_desc *desc, int n, int h, int w);
int cnncrf_net_destroy(cnncrf_net_t net);
/* Stream all later work of this net is enqueued on. */
int cnncrf_net_set_stream(cnncrf_net_t net, cnncrf_stream_t stream);

/* StereoNet::initNet(min, max, step, rect_corr, d_unaryOut, d_pairwiseOut)
 * (stereo/stereonet.h:43-44, stereo/stereonet.cpp:65-182).  d_unary_out is a
 * caller-owned H x W x D volume (may be NULL: owned internally); d_pairwise_out
 * a caller-owned [2][H][W] buffer (may be NULL).  rect_corr must be 0. */
int cnncrf_net_init(cnncrf_net_t net, float min_disp, float max_disp, float step, int rect_corr,
                    float *d_unary_out, float *d_pairwise_out);

/* StereoNet::setAllParams(npzPath) (stereo/stereonet.cpp:184-227): arrays
 * arr_0.. in op order, shapes checked (ESHAPE instead of exit(-1),
 * stereo/operators/operator.cpp:72-79).  Reads STORED and DEFLATE members. */
int cnncrf_net_set_all_params(cnncrf_net_t net, const char *npz_path);

/* Operator::setParams(h_params) for one array (stereo/operators/operator.cpp:87-102).
 * index = the arr_<index> slot; shape as in the npz (4-D filter or 1-D bias). */
int cnncrf_net_set_param(cnncrf_net_t net, int index, const float *h_data, const int64_t *shape,
                         int ndim);
/* Host-side npz access (no device work; the reference's cnpy::npz_load,
 * stereo/operators/operator.cpp:55-85, and a writer it does not have).
 * cnncrf_npz_read: member `key` (".npy" appended) of a STORED or DEFLATE
 * archive of little-endian float32 C-order arrays; fills shape[0..ndim-1]
 * (ndim <= 4, else ESHAPE) and, when h_data is not NULL, copies the values
 * (capacity in floats; ESHAPE when too small).  EIO for a missing file or
 * member.  cnncrf_npz_write: `count` members keys[i] of shapes
 * shapes[4 i .. 4 i + ndims[i] - 1] from host arrays, uncompressed (numpy.load
 * reads it), written beside `npz_path` and renamed over it. */
int cnncrf_npz_read(const char *npz_path, const char *key, int64_t shape[4], int *ndim, float *h_data,
                    size_t capacity);
int cnncrf_npz_write(const char *npz_path, int count, const char *const *keys, const float *const *h_data,
                     const int64_t *shapes, const int *ndims);
/* Number of parameter arrays (filters + biases) the net expects. */
int cnncrf_net_num_params(cnncrf_net_t net, int *count);
/* Shape of arr_<index>. */
int cnncrf_net_param_shape(cnncrf_net_t net, int index, int64_t shape[4], int *ndim);
/* Xavier-uniform filters from a seeded generator, zero biases (no reference
 * counterpart: the synthetic-weight workloads use it). */
int cnncrf_net_init_xavier(cnncrf_net_t net, uint64_t seed);

/* StereoNet::setDisparities(min, max, step, d_out) (stereo/stereonet.cpp:229-248,
 * stereo/operators/stereocorrelation.cpp:71-144): the list is built as
 * `for (d = min; d <= max; d += step)` in float. */
int cnncrf_net_set_disparities(cnncrf_net_t net, float min_disp, float max_disp, float step,
                               float *d_out);
int cnncrf_net_num_disparities(cnncrf_net_t net, int *num);

/* ColorStereoNet::predict(d_left, d_right) (stereo/colorstereonet.cpp:38-77):
 * padded RGBA device images (h x w as created) -> H x W x D unary volume
 * (H = h - 2*pad, W = w - 2*pad), returned as a non-owned device pointer;
 * the pairwise weights (if built) land in the pairwise buffer. */
int cnncrf_net_predict(cnncrf_net_t net, const float *d_left_rgba, const float *d_right_rgba,
                       float **d_volume);
/* Device pointer of the [2][H][W] pairwise output (|conv|, before lambda). */
int cnncrf_net_pairwise(cnncrf_net_t net, float **d_pairwise);
/* Copy the final feature maps of one side (0 left, 1 right) as FP32
 * H x W x C (C = feat_channels) into d_out (debug / parity). */
int cnncrf_net_features(cnncrf_net_t net, int side, float *d_out);
/* Mirror padding amount the topology needs (stereo/stereo.cpp:204-217). */
int cnncrf_net_padding(cnncrf_net_t net, int *pad);

/* ---------------------------------------------------------------- operators */

/* StereoCorrelation::forward(d_input0, d_input1, d_disparities, d_output, in,
 * ic, ih, iw, lenDisps, layout, rectCorr) (stereo/operators/stereocorrelation.cpp:146-152,
 * stereo/operators/stereocorrelation.cu:358-408): NCHW feature inputs, NHWC
 * output, disparity list given as stored by the reference (negated values).
 * The fractional-disparity (interpolating) kernel is chosen exactly when the
 * reference chooses it.  FP32, rect_corr must be 0. */
int cnncrf_correlation_forward(const float *d_input0, const float *d_input1,
                               const float *h_disparities, float *d_output, int n, int c, int h,
                               int w, int num_disps, cnncrf_stream_t stream);

/* ---------------------------------------------------------------- CRF */

typedef struct cnncrf_crf_options {
    float L1;       /* ops["L1"] */
    float L2;       /* ops["L2"] */
    float delta;    /* ops["delta"]: rho's window, integer 1..8 */
    int total_it;   /* ops["total_it"]: horizontal+vertical passes */
    int shape;      /* cnncrf_pairwise_shape */
    float slack;    /* fraction of a subproblem's slack handed over per pass, (0,1] */
} cnncrf_crf_options;

/* Defaults: L1 1, L2 12, delta 2, total_it 4 (stereo/stereo_img.cpp:78-81), STEP shape, slack 0.5. */
int cnncrf_crf_default_options(cnncrf_crf_options *opt);

/* Device workspace one solve needs (bytes). */
int cnncrf_crf_workspace_size(int width, int height, int depth, size_t *bytes);

/* slack_prop_2D_alg: init(C{K,W,H}, sols) + ops + update_W(wx, wy) + execute()
 * + LB() (call sites stereo/stereo.cpp:140-154, stereo/operators/slackprop.cpp:111-139).
 * d_cost: H x W x D; d_wx, d_wy: H x W (>= 0); d_labels: H x W int32 output.
 * lower_bound: host, may be NULL (the FP64 dual bound after the last pass).
 * d_workspace >= cnncrf_crf_workspace_size bytes, 256-byte aligned. */
int cnncrf_crf_solve(const float *d_cost, const float *d_wx, const float *d_wy, int width,
                     int height, int depth, const cnncrf_crf_options *opt, int32_t *d_labels,
                     double *lower_bound, void *d_workspace, size_t workspace_bytes,
                     cnncrf_stream_t stream);

/* No counterpart in the reference.  The same solve as cnncrf_crf_solve
 * (same arguments, results and errors) with no workspace argument: the
 * scratch lives in a 64 MiB array compiled into this library, and no call
 * allocates device memory.  For callers that may not call cudaMalloc: a
 * plug-in whose host framework owns every device allocation, or a real-time
 * loop that cannot afford a device-wide allocation stall.
 * Limit: cnncrf_crf_workspace_size(width, height, depth) <= 64 MiB (about
 * 8 million labels W*H*D); larger problems return CNNCRF_EINVAL.
 * Errors are checked in cnncrf_crf_solve's order: the options first, then the
 * sizes.  The first call in each CUDA context (per device, and again after a
 * reset of the device's primary context) looks up the array's address and
 * caches it; make that first call before any stream capture: a first call on
 * a capturing stream returns CNNCRF_ESTATE.
 * Nothing in the array has to start at zero.  All calls on a device share the
 * one array: calls that overlap on the GPU (other streams, other threads)
 * race and must be serialised by the caller. */
int cnncrf_crf_solve_static(const float *d_cost, const float *d_wx, const float *d_wy, int width,
                            int height, int depth, const cnncrf_crf_options *opt, int32_t *d_labels,
                            double *lower_bound, cnncrf_stream_t stream);

/* CRF tiles.  No counterpart in the reference, whose solver has one launch
 * shape.  A tile is the chain kernel's prefetch ring depth (4 or 8 chain
 * steps) and chains per CTA (1, 2 or 4) for the horizontal and the vertical
 * pass.  Every tile gives the same labels and bound bit for bit; the fastest
 * depends on the label count, the chain lengths and the pairs per launch, so
 * the library keeps a process-wide table from (width, height, depth, npairs,
 * delta) to a tile.  Every solve (cnncrf_crf_solve, SlackProp, Stereo, the
 * batch) looks its shape up and runs the default tile (ring 8, 2 chains per
 * CTA, both passes) when the table has none.  The table is filled by the two
 * autotune calls below or set by hand, and can be saved to a text file and
 * merged back, so a deployment measures once.  Thread-safe. */
typedef struct cnncrf_crf_tile {
    int ring_h, chains_per_cta_h; /* horizontal pass */
    int ring_v, chains_per_cta_v; /* vertical pass */
} cnncrf_crf_tile;
int cnncrf_crf_tuning_set(int width, int height, int depth, int npairs, int delta, const cnncrf_crf_tile *tile);
/* *found = 0 and the default tile when the table has no entry; ms_h / ms_v
 * (may be NULL): the pass times the autotuner measured, 0 for a set tile. */
int cnncrf_crf_tuning_get(int width, int height, int depth, int npairs, int delta, cnncrf_crf_tile *tile,
                          int *found, float *ms_h, float *ms_v);
int cnncrf_crf_tuning_clear(void);
int cnncrf_crf_tuning_count(int *n);
/* Text file: the line "cnncrf-crf-tiles 1", then one line per entry
 * "W H D npairs delta ring_h chains_h ring_v chains_v ms_h ms_v"; '#' starts
 * a comment line.  Load merges into the table; a malformed file returns
 * CNNCRF_EINVAL naming the line and changes nothing. */
int cnncrf_crf_tuning_save(const char *path);
int cnncrf_crf_tuning_load(const char *path);
/* Measures every tile on this problem (one horizontal and one vertical pass
 * each, best of three, CUDA events on `stream`) and enters the fastest per
 * pass for (width, height, depth, 1, opt->delta).  Arguments as
 * cnncrf_crf_solve; the workspace's contents are overwritten (the next solve
 * does not depend on them).  Synchronises the stream: not during a capture. */
int cnncrf_crf_autotune(const float *d_cost, const float *d_wx, const float *d_wy, int width, int height,
                        int depth, const cnncrf_crf_options *opt, void *d_workspace, size_t workspace_bytes,
                        cnncrf_stream_t stream);

/* Object form of the same solver, mirroring slack_prop_2D_alg's members. */
typedef struct cnncrf_slackprop *cnncrf_slackprop_t;
int cnncrf_slackprop_create(cnncrf_slackprop_t *sp);
int cnncrf_slackprop_destroy(cnncrf_slackprop_t sp);
int cnncrf_slackprop_set_stream(cnncrf_slackprop_t sp, cnncrf_stream_t stream);
/* init(ndarray_ref<float,3> C{K,W,H}, ndarray_ref<int,2> sols) */
int cnncrf_slackprop_init(cnncrf_slackprop_t sp, const float *d_cost, int width, int height,
                          int depth, int32_t *d_labels);
/* ops["L1"|"L2"|"delta"|"total_it"|"slack"|"shape"] = value */
int cnncrf_slackprop_set_op(cnncrf_slackprop_t sp, const char *name, double value);
/* update_W(wx, wy) */
int cnncrf_slackprop_update_w(cnncrf_slackprop_t sp, const float *d_wx, const float *d_wy);
/* execute() */
int cnncrf_slackprop_execute(cnncrf_slackprop_t sp);
/* LB() */
int cnncrf_slackprop_lower_bound(cnncrf_slackprop_t sp, double *lb);
/* get_C1(): device pointer to the H x W x D unary share of the horizontal
 * subproblem after the last pass (the reparametrised volume). */
int cnncrf_slackprop_get_c1(cnncrf_slackprop_t sp, float **d_c1);

/* cuda::remapSolution (stereo/stereo.cu:841-850,1229-1246): disp = label*step + min. */
int cnncrf_remap_solution(float *d_out, const int32_t *d_labels, int width, int height,
                          float disp_min, float disp_step, cnncrf_stream_t stream);

/* ---------------------------------------------------------------- refinement */

/* warp_image_kernel (stereo/stereo.cu:830-839): out(x,y) = in(floor(x+0.5-u), y),
 * index clamped to the image (point sampling, clamp addressing). */
int cnncrf_warp_image(float *d_out_rgba, const float *d_in_rgba, const float *d_u, int width,
                      int height, cnncrf_stream_t stream);
/* do_fitting_kernel (stereo/stereo.cu:419-442, do_abs = false): H x W x 3
 * volume -> qf, H x W x 2 interleaved (a, b) like ImageGpu_32f_C2. */
int cnncrf_tv_fit(const float *d_volume3, float *d_qf, int width, int height, float disp_step,
                  float lambda_census, cnncrf_stream_t stream);
/* The inner loop of cuda::fuseTHuberQuadFit (stereo/stereo.cu:1133-1135,1159-1166):
 * p = q = 0, then `iterations` x (u_ = u; primal; dual) with tau = sigma = 1/sqrt(8).
 * d_u, d_u_, d_u0: H x W; d_qf, d_p, d_q: H x W x 2; huber_eps = 0.1 in the
 * reference (stereo/stereo.cu:792).  The iterations run fused, several per
 * launch on tiles held on chip (the results equal the reference's
 * per-iteration passes), and need a device workspace of
 * cnncrf_tv_workspace_size bytes, 256-byte aligned; u, u_, p and q hold the
 * final state on return. */
int cnncrf_tv_workspace_size(int width, int height, size_t *bytes);
int cnncrf_tv_iterate(float *d_u, float *d_u_, const float *d_u0, const float *d_qf, float *d_p,
                      float *d_q, const float *d_wx, const float *d_wy, int width, int height,
                      float C, float huber_eps, float disp_step, int iterations,
                      void *d_workspace, size_t workspace_bytes, cnncrf_stream_t stream);

/* ---------------------------------------------------------------- census, edges, QuadDirect, LR */

/* rgb_to_gray_kernel (stereo/stereo.cu:853-863): .2989 R + .5870 G + .1140 B. */
int cnncrf_rgb_to_gray(const float *d_rgba, float *d_gray, int width, int height, cnncrf_stream_t stream);
/* cost_vol_census_kernel (stereo/stereo.cu:306-346): H x W x depth volume;
 * disparity z = disp_min + z*disp_step (float accumulation), the census window
 * (2 filter_size + 1)^2 without its centre, value = lambda * mismatches /
 * (4 filter_size^2).  Grey images are read clamp-addressed; at fractional
 * disparities linearly interpolated in FP32.  Synchronises the stream. */
int cnncrf_census_volume(const float *d_gray_ref, const float *d_gray_other, int width, int height,
                         int filter_size, float disp_min, float disp_step, int depth, float lambda,
                         float *d_volume, cnncrf_stream_t stream);
/* calcEdgeImage (stereo/stereo.cu:1090-1095, 471-520): Gaussian (sigma 0.7,
 * radius 3, clamp-to-edge) of the grey image, forward differences, then
 * w = alpha > 0 ? max(lambda exp(-alpha |d|^beta), 1e-6) : lambda |d|.
 * Synchronises the stream. */
int cnncrf_edge_weights(const float *d_gray, int width, int height, float alpha, float beta, float lambda,
                        float *d_wx, float *d_wy, cnncrf_stream_t stream);
/* fuseQuadFitDirect (stereo/stereo.cu:913-942, 1172-1194): per pixel the
 * parabola through the costs of labels z-1, z, z+1 of d_c1 (H x W x depth)
 * around z = (int)((u - disp_min) / disp_step); u += (c0 - c2) / (2 h) /
 * max(1e-3, (c0 + c2 - 2 c1) / h^2).  Pixels at z <= 0 or z >= depth - 1 are
 * left unchanged. */
int cnncrf_quad_fit_direct(float *d_u, const float *d_c1, int width, int height, int depth,
                           float disp_min, float disp_step, cnncrf_stream_t stream);
/* leftrightcheck_kernel (stereo/stereo.cu:803-817): out = d if |d - (-right(x - d))| <= th,
 * else -1 (right read clamp-addressed, linear in x). */
int cnncrf_left_right_check(const float *d_left, const float *d_right, int width, int height,
                            float threshold, float *d_out, cnncrf_stream_t stream);

/* ---------------------------------------------------------------- training step */

/* No counterpart in the reference, which ships inference only.  One step of
 * end-to-end training of the feature net and the pairwise net through the
 * CRF: the forward keeps every layer's activations (FP32); the structured
 * hinge with margin 1 per mislabelled pixel takes the CRF's labelling y^ of
 * the loss-augmented energy (the unary plus 1 at each ground-truth label):
 *   loss = E(gt) - E(y^) + #(y^ != gt),
 *   E(y) = sum_i vol[i][y_i] + sum_edges lambda pw rho(|y_i - y_j|);
 * its subgradient (+1 at gt, -1 at y^ in the volume; lambda (rho(gt) -
 * rho(y^)) per edge) goes back through the hand-written adjoints of the
 * correlation, the L2 normalisation, the tanh convolutions and the |1x1|
 * head into every parameter; SGD with momentum (v = mu v + g, theta -= lr v)
 * updates FP32 master weights in the npz layout (stereo/stereonet.cpp:191-223).
 * Nets: num_layers 3x3 (or reference-topology) tanh layers, one-minus-dot
 * unary, integer disparity list, RGB; images [npairs][height][width][4] RGBA
 * on the device, mirror-padded and normalised inside as in predict.
 * Recomputation changes no result bit: a checkpointed step equals the
 * keep-all step exactly. */
typedef struct cnncrf_train *cnncrf_train_t;

typedef struct cnncrf_train_desc {
    int num_layers;     /* 7 */
    int topology;       /* CNNCRF_TOPO_ALL3X3 (default) or CNNCRF_TOPO_REF */
    int feat_channels;  /* 100 */
    int pw_channels;    /* 64 */
    float disp_min, disp_step, disp_max; /* integer disparities disp_min + k step <= disp_max: 0, 1, 127 */
    float lambda;       /* w = lambda * |pairwise net|: 1 */
    float L1, L2;       /* rho: 0.5, 1.5 */
    int delta;          /* 3 */
    int crf_shape;      /* CNNCRF_RHO_LINEAR */
    float crf_slack;    /* 0.5 */
    int crf_iters;      /* 8 */
    int mean_loss;      /* 1: per-pair losses per pixel, the gradient of their mean over the batch
                           (the scale at which lr 1e-3 is a sane step); 0: plain sums */
    int precision;      /* CNNCRF_BF16 (default): tensor-core forward, BF16 activations, FP32 gradients
                           and master weights; CNNCRF_FP32: the exact path (forward equals the oracle's) */
    int checkpoint_every; /* r > 0 (default 3): keep every r-th feature layer's output and the last,
                             recompute the others during backward; 0: keep all */
    int tc_wgrad;       /* BF16 mode: 1 (default) the weight gradients of layers with 16..128 input
                           channels on the tensor cores (dz rounded to BF16); 0: on the CUDA cores (FP32 dz) */
    int tc_dgrad;       /* BF16 mode: 1 (default) the input gradients of those layers on the tensor cores
                           (dz rounded to BF16, FP32 sums); 0: on the CUDA cores */
} cnncrf_train_desc;

int cnncrf_train_default_desc(cnncrf_train_desc *d);
int cnncrf_train_create(cnncrf_train_t *t, const cnncrf_train_desc *d, int npairs, int width, int height);
int cnncrf_train_destroy(cnncrf_train_t t);
int cnncrf_train_set_stream(cnncrf_train_t t, cnncrf_stream_t stream);
/* parameters in the npz slot order of cnncrf_net_set_param, npz shapes */
int cnncrf_train_num_params(cnncrf_train_t t, int *n);
int cnncrf_train_param_shape(cnncrf_train_t t, int i, int64_t shape[4], int *ndim);
int cnncrf_train_init_xavier(cnncrf_train_t t, uint64_t seed); /* the nets' seeded Xavier init; momentum zeroed */
/* host or device pointers; count = the slot's element count (else CNNCRF_ESHAPE) */
int cnncrf_train_set_param(cnncrf_train_t t, int i, const float *data, size_t count);
int cnncrf_train_get_param(cnncrf_train_t t, int i, float *data, size_t count);
int cnncrf_train_get_grad(cnncrf_train_t t, int i, float *data, size_t count);
/* forward: the unary volume [npairs][H][W][D] and the pairwise output |h|
 * (before lambda) [npairs][2][H][W] stay on the device (cnncrf_train_outputs) */
int cnncrf_train_forward(cnncrf_train_t t, const float *d_left, const float *d_right);
int cnncrf_train_outputs(cnncrf_train_t t, const float **d_volume, const float **d_pairwise, int *depth);
/* after forward: the loss-augmented CRF solve, the loss of every pair
 * (h_loss[npairs], may be NULL) and the subgradient; d_gt [npairs][H][W]
 * labels in 0..D-1 (CNNCRF_EINVAL otherwise); d_labels (may be NULL): y^.
 * Synchronises the stream. */
int cnncrf_train_hinge(cnncrf_train_t t, const int32_t *d_gt, double *h_loss, int32_t *d_labels);
/* the hinge's subgradient buffers ([npairs][H][W][D] and [npairs][2][H][W])
 * of the last cnncrf_train_hinge, valid until the next forward */
int cnncrf_train_hinge_grads(cnncrf_train_t t, const float **d_gvol, const float **d_gpw);
/* After a forward: measures the CRF tiles on the hinge's problem (the unary and the weighted pairwise output,
 * all npairs crops in one solve) and enters the fastest per pass in the process-wide tile table, where every
 * later hinge of this shape finds it.  Tiles change no bit.  Synchronises the stream. */
int cnncrf_train_autotune(cnncrf_train_t t);
/* parameter gradients of sum(gvol * vol) + sum(gpw * pw) (gpw may be NULL:
 * the pairwise net gets none), or of the hinge loss when both are NULL */
int cnncrf_train_backward(cnncrf_train_t t, const float *d_gvol, const float *d_gpw);
int cnncrf_train_sgd(cnncrf_train_t t, float lr, float momentum);
/* forward + hinge + backward + sgd */
int cnncrf_train_step(cnncrf_train_t t, const float *d_left, const float *d_right, const int32_t *d_gt, float lr,
                      float momentum, double *h_loss);
/* Training checkpoint (no counterpart in the reference, which has no save
 * path and no training state; its weights load through cnpy, stereo/operators/
 * operator.cpp:55-85).  Save writes an uncompressed npz: arr_0 .. arr_{n-1},
 * the FP32 master weights in the slot order and shapes of
 * cnncrf_net_set_all_params, so the file is also a parameter file for
 * inference (cnncrf_net_set_all_params, Stereo's parameter-file); and
 * mom_0 .. mom_{n-1}, the SGD momentum.  The file is written beside `path`
 * and renamed over it.  Load reads arr_i (shapes checked: ESHAPE) and mom_i
 * when present (zero momentum when absent, so a plain parameter file starts
 * a fresh run from those weights).  A loaded trainer continues bit for bit
 * as the saved one would have.  Both synchronise the trainer's stream. */
int cnncrf_train_save(cnncrf_train_t t, const char *npz_path);
int cnncrf_train_load(cnncrf_train_t t, const char *npz_path);

/* ---------------------------------------------------------------- Stereo */

typedef struct cnncrf_stereo *cnncrf_stereo_t;

typedef struct cnncrf_stereo_options {
    int precision;       /* cnncrf_precision (default FP32) */
    int unary;           /* cnncrf_unary (default NEG_SOFTMAX) */
    int topology;        /* cnncrf_topology (default REF) */
    int feat_channels;   /* 100 */
    int pw_channels;     /* 64 */
    int ref_depth_rounding; /* 1: depth -> min(256, next pow2) as stereo/stereo.cpp:71-73 */
    int crf_shape;       /* cnncrf_pairwise_shape (default STEP) */
    float crf_slack;     /* default 0.5 */
    float huber_eps;     /* default 0.1 (stereo/stereo.cu:792) */
    int refine_interp;   /* 0: the reference's 3-label dispatch; 1: always interpolate */
} cnncrf_stereo_options;

int cnncrf_stereo_default_options(cnncrf_stereo_options *opt);
/* Stereo() (stereo/stereo.h:43) */
int cnncrf_stereo_create(cnncrf_stereo_t *s, const cnncrf_stereo_options *opt);
int cnncrf_stereo_destroy(cnncrf_stereo_t s);
int cnncrf_stereo_set_stream(cnncrf_stereo_t s, cnncrf_stream_t stream);
/* Stereo::initialize(size, disp_min, disp_step, disp_max) (stereo/stereo.cpp:64-105) */
int cnncrf_stereo_initialize(cnncrf_stereo_t s, int width, int height, float disp_min,
                             float disp_step, float disp_max);
/* setMatchingFunction / setNumLayers / setParameterFile / setWithXy
 * (stereo/stereo.h:52-54,82).  The parameter file gets ".npz" appended
 * (stereo/stereo.cpp:188).  Pass NULL to keep Xavier weights (seed). */
int cnncrf_stereo_set_matching_function(cnncrf_stereo_t s, int matching);
int cnncrf_stereo_set_num_layers(cnncrf_stereo_t s, int num_layers);
int cnncrf_stereo_set_parameter_file(cnncrf_stereo_t s, const char *base_name);
int cnncrf_stereo_set_xavier_seed(cnncrf_stereo_t s, uint64_t seed);
int cnncrf_stereo_set_with_xy(cnncrf_stereo_t s, int with_xy);
/* Stereo::setColorImages(ImageCpu_32f_C4 x2) (stereo/stereo.cpp:117-126): host RGBA. */
int cnncrf_stereo_set_color_images(cnncrf_stereo_t s, const float *h_left_rgba,
                                   const float *h_right_rgba);
/* Same with device RGBA buffers (device-to-device copy). */
int cnncrf_stereo_set_color_images_device(cnncrf_stereo_t s, const float *d_left_rgba,
                                          const float *d_right_rgba);
/* Stereo::computeVolume(lr) (stereo/stereo.cpp:179-318) */
int cnncrf_stereo_compute_volume(cnncrf_stereo_t s, int lr);
/* Stereo::computeSlackPropagation(C1, C2, delta, iterations, alpha, beta,
 * lambda, lr) (stereo/stereo.cpp:129-162).  Pairwise (COLORPAIR) matching
 * uses the pairwise CNN's weights times lambda; every other matching the
 * image-gradient edge weights of (alpha, beta, lambda). */
int cnncrf_stereo_compute_slack_propagation(cnncrf_stereo_t s, float C1, float C2, float delta,
                                            int iterations, float alpha, float beta,
                                            float lambda_reg, int lr);
/* Stereo::setFilterSize (census window half-size, stereo/stereo_img.cpp:73, default 7). */
int cnncrf_stereo_set_filter_size(cnncrf_stereo_t s, int filter_size);
/* Stereo::computeWeights(alpha, beta, lambda, lr) (stereo/stereo.cpp:320-326):
 * edge weights of the reference side's grey image into the wx / wy buffers. */
int cnncrf_stereo_compute_weights(cnncrf_stereo_t s, float alpha, float beta, float lambda_reg, int lr);
/* Stereo::fuseQuadFitDirect() (stereo/stereo.cpp:406-409): QuadDirect on the
 * solver's get_C1() volume after computeSlackPropagation. */
int cnncrf_stereo_fuse_quad_fit_direct(cnncrf_stereo_t s);
/* Stereo::computeArgMax(lr) (stereo/stereo.cpp:164-177; arg_min_kernel stereo/stereo.cu:348-370) */
int cnncrf_stereo_compute_argmax(cnncrf_stereo_t s, int lr);
/* Stereo::fuseTHuberQuadFit(lambda, C, iterations, warps) (stereo/stereo.cpp:388-404) */
int cnncrf_stereo_fuse_thuber_quad_fit(cnncrf_stereo_t s, float lambda_reg, float C,
                                       int iterations, int warps);
/* Stereo::getOutput() (stereo/stereo.cpp:412-417): H x W float disparity. */
int cnncrf_stereo_get_output(cnncrf_stereo_t s, float *h_out);
int cnncrf_stereo_get_output_device(cnncrf_stereo_t s, const float **d_out);
/* Stereo::getIntegerOutput() (stereo/stereo.cpp:439-442) */
int cnncrf_stereo_get_labels_device(cnncrf_stereo_t s, const int32_t **d_labels);
/* Stereo::getVolume() (stereo/stereo.cpp:419-423) */
int cnncrf_stereo_get_volume_device(cnncrf_stereo_t s, const float **d_volume);
/* Stereo::getWx / getWy (stereo/stereo.cpp:425-437): lambda-scaled weights. */
int cnncrf_stereo_get_weights_device(cnncrf_stereo_t s, const float **d_wx, const float **d_wy);
/* Stereo::getDepth() (stereo/stereo.cpp:444-447) */
int cnncrf_stereo_get_depth(cnncrf_stereo_t s, int *depth);
/* The solver's LB() after the last computeSlackPropagation. */
int cnncrf_stereo_lower_bound(cnncrf_stereo_t s, double *lb);
/* Device time of the stages of the last run (CUDA events, ms): cnn, corr,
 * crf, refine; any may be NULL. */
int cnncrf_stereo_stage_times(cnncrf_stereo_t s, float *cnn_ms, float *corr_ms, float *crf_ms,
                              float *refine_ms);

/* ---------------------------------------------------------------- batched Stereo
 * Many pairs through computeSlackPropagation at once (no counterpart in the
 * reference: its Stereo object holds one pair, stereo/stereo.h:40-133).
 * Pairs of equal size and disparity range form a group that runs as one
 * batch (tensor-core convolutions over all its images, one correlation and
 * one CRF launch per pass over all its chains); groups run on their own
 * streams, forked from and joined into the batch's stream.  With graph
 * capture on, the first run executes eagerly, the second captures the whole
 * step into a CUDA graph, later runs with the same CRF parameters replay it. */
typedef struct cnncrf_batch *cnncrf_batch_t;
int cnncrf_batch_create(cnncrf_batch_t *b, const cnncrf_stereo_options *opt);
int cnncrf_batch_destroy(cnncrf_batch_t b);
int cnncrf_batch_set_stream(cnncrf_batch_t b, cnncrf_stream_t stream);
/* matching (COLORPAIR / GRAYPAIR), layers, xy channels, weights: npz base
 * name (".npz" appended) or NULL for Xavier weights from `seed`. */
int cnncrf_batch_set_network(cnncrf_batch_t b, int matching, int num_layers, int with_xy,
                             const char *param_base, uint64_t seed);
/* Most pairs per group (0, the default: every pair of one size and range in
 * one group).  Smaller groups pipeline: the CNN of one group runs while the
 * CRF of the previous one streams its volume.  Call before the first
 * add_pair (ESTATE after). */
int cnncrf_batch_set_group_size(cnncrf_batch_t b, int max_pairs);
/* Stereo::initialize for one more pair; returns its index. */
int cnncrf_batch_add_pair(cnncrf_batch_t b, int width, int height, float disp_min, float disp_step,
                          float disp_max, int *pair_index);
int cnncrf_batch_num_pairs(cnncrf_batch_t b, int *n);
/* Stereo::setColorImages for one pair (host RGBA / device RGBA). */
int cnncrf_batch_set_images(cnncrf_batch_t b, int pair, const float *h_left, const float *h_right);
int cnncrf_batch_set_images_device(cnncrf_batch_t b, int pair, const float *d_left,
                                   const float *d_right);
int cnncrf_batch_use_graph(cnncrf_batch_t b, int enable);
/* computeSlackPropagation(L1, L2, delta, iterations, -, -, lambda, lr = 1)
 * for every pair; asynchronous on the batch's stream. */
int cnncrf_batch_run(cnncrf_batch_t b, float L1, float L2, float delta, int iterations,
                     float lambda_reg);
/* cnncrf_batch_run with the images taken from and the disparities returned to
 * host memory as part of the pipeline (no reference counterpart: Stereo's
 * setColorImages / getOutput, stereo/stereo.cpp:117-126,412-416, per pair).
 * h_left[i], h_right[i]: pair i's RGBA images (H x W x 4 floats); h_out[i]:
 * pair i's H x W disparities, or h_out / h_out[i] NULL for none.  Each group's
 * host-to-device copies run ahead of its CNN on a copy stream, its
 * device-to-host copies right after its remap, so copies overlap the other
 * groups' work.  Asynchronous: h_out holds the results once the batch's
 * stream is synchronised (cnncrf_batch_check).  Graph replay needs the same
 * buffers as the captured run and page-locked ones; other calls run eagerly. */
int cnncrf_batch_run_host(cnncrf_batch_t b, const float *const *h_left, const float *const *h_right,
                          float *const *h_out, float L1, float L2, float delta, int iterations,
                          float lambda_reg);
int cnncrf_batch_get_output(cnncrf_batch_t b, int pair, float *h_out);
int cnncrf_batch_get_output_device(cnncrf_batch_t b, int pair, const float **d_out);
int cnncrf_batch_get_labels_device(cnncrf_batch_t b, int pair, const int32_t **d_labels);
/* The pair's FP32 cost volume.  In BF16 the batch's correlation writes, by
 * default, only the 16-bit fixed-point copy its CRF reads (x = q * 2^-15 - 2^-8
 * for the 1 - <fL,fR> unary, q * 2^-16 - 1 for -softmax, where D / 32 is even);
 * the FP32 volume is then not written and this returns CNNCRF_ESTATE unless
 * cnncrf_batch_keep_volume(b, 1) was set before the run. */
int cnncrf_batch_get_volume_device(cnncrf_batch_t b, int pair, const float **d_volume, int *depth);
int cnncrf_batch_keep_volume(cnncrf_batch_t b, int enable);
int cnncrf_batch_lower_bound(cnncrf_batch_t b, int pair, double *lb);
/* Synchronise and report a kernel that gave up on a bounded wait (ETIMEOUT). */
int cnncrf_batch_check(cnncrf_batch_t b);
/* No counterpart in the reference.  Runs the batch once (the staged images
 * through the whole path), then tunes the CRF tile of every group on its
 * volume (cnncrf_crf_autotune per group, npairs = the group's pairs) and
 * drops the captured graph so the next run captures the tuned launches.  The
 * outputs of that run stay readable.  Synchronises: not during a capture. */
int cnncrf_batch_autotune(cnncrf_batch_t b, float L1, float L2, float delta, int iterations, float lambda_reg);
/* The groups the pairs fall into (same size and range, at most the group
 * size set by cnncrf_batch_set_group_size), in pipeline order. */
int cnncrf_batch_num_groups(cnncrf_batch_t b, int *n);
int cnncrf_batch_group_shape(cnncrf_batch_t b, int group, int *width, int *height, int *depth, int *npairs);

/* ---------------------------------------------------------------- instrumentation
 * (no counterpart in the reference, which timed whole stages with
 * iu::IuCudaTimer when verbose, stereo/stereonet.cpp:258-315) */

/* Number of kernels this library has launched in the process. */
int cnncrf_kernel_launches(uint64_t *count);
/* While enabled, every launch is bracketed by CUDA events on its stream. */
int cnncrf_profile_enable(int enable);
int cnncrf_profile_reset(void);
/* Launches and summed device time (ms) of one kernel since the last reset;
 * synchronises on the recorded events. */
int cnncrf_profile_query(const char *kernel, int *launches, double *total_ms);
/* Newline-separated names of the kernels timed since the last reset. */
int cnncrf_profile_kernels(char *buf, size_t len);

/* No counterpart in the reference (its kernels have no device-side waits).
 * Self-test of the bounded waits and of the error path they feed: one warp
 * waits on a shared-memory mbarrier through the same bounded wait the
 * tensor-core kernels use, giving up after `polls` polls (1 .. 2^20).  With
 * arrive != 0 the barrier completes before the wait and the call returns
 * CNNCRF_OK; with arrive == 0 nothing completes it, the wait runs out, the
 * kernel raises its error flag and the call returns CNNCRF_ETIMEOUT.  The
 * probe moves no data and holds no tensor memory, so the context stays usable
 * after a timeout.  Synchronises the stream. */
int cnncrf_selftest_bounded_wait(int polls, int arrive, cnncrf_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* CNNCRF_H */
