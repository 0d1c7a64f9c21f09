/*
 * cnncrf_oracle.h -- TEST INFRASTRUCTURE, not part of the product.
 *
 * CPU restatement (C++17 + OpenMP) of the reference's CNN-CRF stereo hot path,
 * used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
 * reference legs as the checker.  The product (libcnncrf.so) never links or
 * calls it.
 *
 * Parity status: the CNN, correlation, softmax, normalisation, padding, remap
 * and TV refinement follow the reference sources line by line (citations in
 * cnncrf_oracle.cpp) and are pinned against independent library
 * implementations of the same operators (tests/golden/make_golden.py).  The
 * correlation, padding, grey conversion, census, argmin, remap, warp,
 * quadratic fit, TV primal-dual iterations, left-right check and QuadDirect
 * are also pinned bit for bit against the reference's own CUDA kernels run on
 * a GPU (tests/golden/ref_kernels.npz, written by make_ref_golden.py).  The
 * CRF solver is an absent third-party dependency (SlackProp, un-vendored
 * submodule, no pinned version): its restatement here follows our own written
 * spec and is PARITY UNPINNED against the reference.
 *
 * The CRF spec and where it comes from.  SlackProp is the solver of
 * A. Shekhovtsov, C. Reinbacher, G. Graber, T. Pock, "Solving Dense Image
 * Matching in Real-Time using Discrete-Continuous Optimization", Computer
 * Vision Winter Workshop 2016 (arXiv:1601.06274).  Taken from that published
 * method (the paper is not in this tree, so no section is quoted):
 *  - the energy: unaries plus pairwise terms on the 4-connected grid;
 *  - the dual decomposition of the grid into horizontal and vertical chain
 *    subproblems that share the unary through a dual variable phi (the
 *    horizontal chains see theta - phi, the vertical ones phi), every chain
 *    solved exactly by min-sum dynamic programming;
 *  - the update: a chain's min-marginals are formed and a fraction of their
 *    excess over the chain's minimum -- the "slack" -- is handed to the other
 *    subproblem, which leaves the chain's minimum unchanged, so the sum of
 *    the chain minima is a lower bound of the energy that never decreases.
 * Our own choices where the published description leaves freedom, or that
 * the reference's call sites (stereo/stereo.cpp:140-154) do not pin:
 *  - the slack fraction handed over per node: 0.5 (option `slack`);
 *  - the schedule: one iteration = a horizontal pass then a vertical pass;
 *    a pass runs the forward messages of every chain, then a backward sweep
 *    that hands over the slack node by node and propagates the reduced unary
 *    backwards, so each node's min-marginal already includes the hand-over
 *    of the nodes after it;
 *  - the bound: the FP64 sum of the last vertical pass's chain minima and of
 *    the horizontal pass before it (the horizontal minima are preserved by
 *    its hand-over, so both are the dual objective at the same phi); a
 *    chain's minimum is the sum of its forward sweep's per-node minima, in
 *    the order the GPU kernel adds them: 32 FP64 partial sums, partial l
 *    taking the nodes i = l mod 32 in ascending i, then added in order; the
 *    chain minima of each direction are summed the same way (partial l over
 *    the chains l, l + 32, ..), and the bound is the H sum plus the V sum;
 *  - the labels: the first argmin of the last vertical pass's min-marginals;
 *  - the pairwise term w_ij rho(|x_i - x_j|): the options L1, L2, delta keep
 *    the reference's names.  STEP (the reference configs' shape): rho(0) = 0,
 *    rho(1..delta) = L1, rho(> delta) = L2 -- the shipped configs
 *    (data/parameters/kitti-2015/7-layer/cnn+crf+full/*.cfg: L1 = 1.002,
 *    L2 = 14.98, delta = 2) then charge L1 for jumps of one or two labels
 *    and L2 for larger ones.  Whether the library reads delta as "<= delta"
 *    or "< delta" is not visible from the reference; "<=" is our reading.
 *    LINEAR: rho(t) = min(L1 t, L2) for t <= delta, L2 beyond (the truncated
 *    linear model of the task's synthetic workloads).
 * Properties the tests check: the chain DP equals brute force; energy >=
 * bound; the bound never decreases; w = 0 gives the winner-take-all labels;
 * ties break to the first minimum; on a problem that is a single chain the
 * bound reaches the minimum energy and the labels are the exact minimiser
 * (the decomposition is exact on trees).  And the bound against the LP
 * relaxation of the energy over the local polytope: a decomposition into
 * trees that cover every edge has that LP's dual as its own (Wainwright,
 * Jaakkola, Willsky, "MAP estimation via agreement on trees", IEEE Trans.
 * Inf. Theory 2005; Komodakis, Paragios, Tziritas, "MRF optimization via dual
 * decomposition", ICCV 2007), so the bound stays at or below the LP optimum
 * at every iteration, and on the tested grids it reaches it: after 200-300
 * iterations it equals the optimum that an LP solver (scipy's HiGHS) finds
 * from the energy alone.  That pins the solver's fixed point -- the bound it
 * converges to -- independently of this restatement's arithmetic.
 *
 * The float instantiation uses exactly the operation order of the GPU FP32
 * path (explicit fmaf, the shared exp/tanh of include/cnncrf_fmath.h), so the
 * GPU output is compared bit for bit; the double instantiation is the FP64
 * oracle the BF16 path's errors are stated against.
 */
#ifndef CNNCRF_ORACLE_H
#define CNNCRF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_cfg {
    /* network */
    int num_layers;
    int topology;      /* 0 ref (3x3 then 2x2), 1 all 3x3, 2 ConcatStereoNet (zero-padded, concatenated) */
    int in_channels;   /* 1, 3, 5 */
    int feat_channels; /* 100 */
    int unary;         /* 0 -softmax, 1 one-minus-dot (L2-normalised features) */
    int with_pairwise;
    int pw_channels; /* 64 */
    int precision;   /* 32 or 64 */
    /* disparities: the reference's float loop list */
    float disp_min, disp_step, disp_max;
    /* CRF */
    float lambda;
    float L1, L2, delta;
    int crf_iters;
    int crf_shape;
    float crf_slack;
    /* refinement (warps == 0: none) */
    int ref_iters, warps;
    float huber_eps;
    float C;
    int refine_interp;
    int threads; /* OpenMP threads, 0 = default */
} oracle_cfg;

/* number of parameter slots and the mirror-pad amount for a cfg */
int oracle_num_params(const oracle_cfg *cfg);
int oracle_padding(const oracle_cfg *cfg);
/* npz shape of slot i */
int oracle_param_shape(const oracle_cfg *cfg, int i, int64_t shape[4], int *ndim);
/* Xavier weights of slot i (cnncrf_xavier.h) */
void oracle_xavier(const oracle_cfg *cfg, int i, uint64_t seed, float *out);

/* mirror pad RGBA (stereo/stereo.cu:879-911) */
void oracle_pad_rgba(const float *in, int W, int H, int p, float *out);
/* pack + zero-mean/unit-std (+xy / gray) of a padded RGBA image -> NHWC planes */
void oracle_normalize(const float *rgba, int Wp, int Hp, int in_channels, int precision,
                      void *out);
/* one valid conv layer, NHWC in/out, weights in npz layout (co,ci,kh,kw);
 * act: 0 none, 1 tanh, 2 abs */
void oracle_conv(const void *in, int H, int W, int Cin, const float *w, const float *b, int Cout,
                 int kh, int kw, int act, int precision, void *out, int threads);
/* per-pixel L2 normalisation of NHWC features */
void oracle_l2norm(void *f, long npx, int C, int precision);
/* raw correlation, NHWC features -> H x W x D (stored disparity list) */
void oracle_correlation(const void *fl, const void *fr, int H, int W, int C, const float *list,
                        int D, int precision, void *out, int threads);
/* -softmax over D in place, or 1 - x (unary = 1) */
void oracle_unary(void *vol, long npx, int D, int unary, int precision);
/* reference disparity list; returns count (<= cap) */
int oracle_disparity_list(float min, float max, float step, float *list, int cap);
/* does the reference pick its interpolating kernel for this list? */
int oracle_disp_is_float(const float *list, int D);

/* full ColorStereoNet::predict on padded RGBA images (h x w padded size).
 * params: array of nparams pointers (npz layout).  vol: H x W x D (float or
 * double per precision), pw: [2][H][W] |conv| (may be NULL). */
int oracle_predict(const oracle_cfg *cfg, const float *const *params, const float *left_pad,
                   const float *right_pad, int w, int h, const float *list, int D, void *vol,
                   void *pw);

/* CRF solve (our SlackProp spec), FP32 messages, FP64 bound.
 * lb_iters: per-iteration bounds (crf_iters entries, may be NULL). */
void oracle_crf(const float *cost, const float *wx, const float *wy, int W, int H, int D,
                float L1, float L2, int delta, int iters, int shape, float slack, int32_t *labels,
                double *lb, double *lb_iters, float *c1_out, int threads);
/* energy of a labelling in FP64 */
double oracle_energy(const float *cost, const float *wx, const float *wy, int W, int H, int D,
                     float L1, float L2, int delta, int shape, const int32_t *labels);
/* brute-force minimum of a single chain (tests): returns min energy, writes labels */
double oracle_chain_bruteforce(const float *cost, const float *w, int n, int D, float L1, float L2,
                               int delta, int shape, int32_t *labels);

/* remap label -> disparity (stereo/stereo.cu:848) */
void oracle_remap(const int32_t *labels, long n, float dmin, float dstep, float *out);
/* grey image, census volume, edge weights, QuadDirect, left-right check
 * (stereo/stereo.cu:853-863, 306-346, 1090-1095, 913-942, 803-817) */
void oracle_gray(const float *rgba, long n, float *gray);
void oracle_census(const float *g1, const float *g2, int W, int H, int fs, const float *list, int D,
                   float lambda, float *vol);
void oracle_gauss_weights(float sigma, int R, float *w);
void oracle_edge_weights(const float *gray, int W, int H, float alpha, float beta, float lambda, float *wx,
                         float *wy);
void oracle_quadfit_direct(float *u, const float *c1, long npx, int D, float dmin, float dstep);
void oracle_lr_check(const float *left, const float *right, int W, int H, float th, float *out);
/* WTA (stereo/stereo.cu:348-370) */
void oracle_argmin(const float *vol, long npx, int D, float dmin, float dstep, float *out);
/* nearest warp (stereo/stereo.cu:830-839) */
void oracle_warp(const float *in_rgba, const float *u, int W, int H, float *out_rgba);
/* quadratic fit (stereo/stereo.cu:419-442) */
void oracle_tv_fit(const float *vol3, int W, int H, float step, float lambda_census, float *qf);
/* primal-dual iterations (stereo/stereo.cu:701-796,1159-1166); p, q zeroed by caller */
void oracle_tv_iterate(float *u, float *u_, const float *u0, const float *qf, float *p, float *q,
                       const float *wx, const float *wy, int W, int H, float C, float eps,
                       float step, int iters);

/* Whole Stereo path for one pair of (unpadded) RGBA images: computeVolume +
 * computeSlackPropagation (+ fuseTHuberQuadFit when cfg->warps > 0).
 * Outputs (any may be NULL): disp H x W, labels H x W, vol H x W x D (float),
 * wx / wy H x W (lambda-scaled), lb. Returns 0 or an error code. */
int oracle_run_pair(const oracle_cfg *cfg, const float *const *params, const float *left,
                    const float *right, int W, int H, float *disp, int32_t *labels, float *vol,
                    float *wx, float *wy, double *lb);

/* Backward of oracle_predict in FP64 (one-minus-dot unary, integer lists):
 * gvol = dL/dvol (H x W x D), gpw = dL/dpw ([2][H][W], may be NULL) -> grads[i],
 * slot i's gradient in its npz layout (doubles, overwritten).  Returns 0, or
 * 3 (unary not one-minus-dot), 4 (fractional list), 1 / 2 (shape). */
int oracle_predict_backward(const oracle_cfg *cfg, const float *const *params, const float *left_pad,
                            const float *right_pad, int w, int h, const float *list, int D,
                            const double *gvol, const double *gpw, double *const *grads);

#ifdef __cplusplus
}
#endif

#endif
