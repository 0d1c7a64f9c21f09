// kernels.h -- host-side launchers of the CUDA kernels of libcnncrf.
// Every launcher enqueues on `st` and returns a cnncrf_status.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/cnncrf.h"

namespace cnncrf {
namespace k {

// ------------------------------------------------------------ front end
// mirror pad of an RGBA image (stereo/stereo.cu:879-911)
int pad_rgba(const float *in, int W, int H, int p, float *out, cudaStream_t st, int nimg = 1);
// zero-mean / unit-std planes of a padded RGBA image -> NHWC [Hp][Wp][ic]
// (stereo/colorstereonet.cpp:53-64,102-121; stereo/utils.cu:169-237).
// scratch: >= 6*Hp doubles + 8 floats.
// images of a batch are contiguous ([nimg][Hp][Wp][4] in, [nimg][Hp][Wp][ic] out)
int normalize(const float *rgba, int Wp, int Hp, int ic, float *out, void *scratch,
              cudaStream_t st, int nimg = 1);
size_t normalize_scratch_bytes(int Hp, int nimg = 1);

// ------------------------------------------------------------ FP32 conv
struct ConvArgs {
    const float *in;
    int H, W, Cin;        // input extent (valid conv)
    long in_pix, in_row;  // element strides of a pixel and of a row
    const float *wt;      // [K][128] flipped, transposed, zero padded
    const float *bias;    // [128] or nullptr
    int Cout, kh, kw, act; // act: 0 none, 1 tanh, 2 abs, 3 |tanh|
    float *out;           // NHWC dense [Ho][Wo][Cout], unless strides are given below
    void *out16 = nullptr; // if set: BF16 NHWC output [Ho][Wo][out_cs] instead of `out`
    int out_cs = 0;
    int n_img = 1;         // images of a batch: input / output element strides
    long in_img = 0, out_img = 0;
    // FP32 output element strides of a pixel, a row and a channel (out_pix = 0:
    // dense NHWC); e.g. a channel slice of a wider tensor, or planar [C][Ho][Wo]
    long out_pix = 0, out_row = 0, out_ch = 1;
};
int conv_simt(const ConvArgs &a, cudaStream_t st);
// BF16 path: a thin first layer (kh*kw*Cin <= 64, Cout 100 or 64, tanh, BF16
// output) on the tensor cores; err: the bounded-wait error flag
bool conv_first_tc_supported(const ConvArgs &a);
int conv_first_tc(const ConvArgs &a, int *err, cudaStream_t st);
// 1x1 conv Cin -> 2, no bias, |.| (stereo/stereonet.cpp:167,401): planar [2][H][W]
int conv_head2(const float *in, int npx, int Cin, const float *w /*[2][Cin]*/, float *out,
               cudaStream_t st, int n_img = 1);
// per-pixel L2 normalisation of NHWC features
int l2norm(float *f, long npx, int C, cudaStream_t st);

// ------------------------------------------------------------ BF16 tensor-core conv
// A tensor-core convolution's launch form: 2-CTA pairs (cta_group::2) or
// single CTAs, and the pipeline stages (0: as many as fit in shared memory).
// Every form gives the same bits; only the speed differs.
struct ConvForm {
    int pair = -1; // -1: the process-wide switch (conv_tc_set_pairs)
    int stages = 0;
};
struct TcConvArgs {
    const void *in; // BF16 NHWC [n_img][Hin][Win][cp_in], channels >= cin zero
    int n_img, Hin, Win, cp_in, cin;
    const void *wt; // BF16 [np][kh*kw][cp_in], kernel flipped
    int np, cout, kh, kw;
    const float *bias; // [np] zero padded
    const float *head; // [2][np] (mode 2)
    int mode;          // 0 tanh -> BF16, 1 tanh + L2 norm -> BF16, 2 tanh + 1x1 head + abs -> FP32 [2][Ho][Wo],
                       // 3 the plain sums -> FP32 [n_img][Ho][Wo][cp_out], channels < cout (input gradients),
                       // 4 the sums times 1 - aux^2 -> FP32 as mode 3 and BF16 into out16 (below)
    void *out;
    int cp_out;
    int *err; // set to 1 if a bounded wait gave up
    // mode 4: aux = BF16 [n_img][Ho][Wo][aux_cs] (the layer below's output); out16 = BF16
    // [n_img][Ho + 2 o16_ph][Wo + 2 o16_pw][o16_cs], written inside its border (channels < np).
    // modes 1 and 2, optional: out16 = the tanh outputs (before the normalisation / the head),
    // [n_img][Ho][Wo][o16_cs]
    const void *aux = nullptr;
    void *out16 = nullptr;
    int aux_cs = 0, o16_cs = 0, o16_ph = 0, o16_pw = 0;
    // mode 4, optional: out (FP32) may be null; bias_part = the per-channel sums of the output, one row
    // of cout floats per (CTA, epilogue warp), *bias_splits = their number (at most 8 x SMs)
    float *bias_part = nullptr;
    int *bias_splits = nullptr;
    ConvForm form; // unset: the tuning table's form for this shape, else the defaults
};
// a.form unset (pair -1, stages 0): the form of the process-wide tuning
// table for this layer shape if it has one, else the switch and the most stages
int conv_tc(const TcConvArgs &a, cudaStream_t st);
// 2-CTA pairs (cta_group::2) for conv_tc where the device co-schedules them (default on)
void conv_tc_set_pairs(bool on);
bool conv_tc_pairs();
// Time every form of this launch (pair or single CTAs x 2..4 stages, best of
// 3, CUDA events on st; synchronises) and enter the fastest in the table.
// Inference modes 0-2 only: the launch's outputs are rewritten, with the same bits.
int conv_tc_autotune(const TcConvArgs &a, cudaStream_t st);
// the conv tuning table: key = n_img, Hin, Win, cp_in, cin, np, cout, kh, kw, mode
constexpr int CONV_KEY = 10;
int conv_forms_count();
bool conv_form_entry(int i, int key[CONV_KEY], ConvForm *f, float *ms);
void conv_forms_clear();

// ------------------------------------------------------------ correlation
// raw correlation (+ unary: -1 none, 0 -softmax, 1 one-minus) of NHWC FP32
// features; list = the reference's stored (negated) disparities.
// npairs pairs: features of pair p at fl + p*fps, fr + p*fps; volume at out + p*H*W*D
int correlation(const float *fl, const float *fr, int H, int W, int C, const float *d_list,
                int D, int omin, int omax, bool interp, int unary, float *out, cudaStream_t st,
                int npairs = 1, long fps = 0);
// same on BF16 features with channel stride cs (FP32 accumulation)
int correlation_bf16(const void *fl, const void *fr, int H, int W, int C, int cs, const float *d_list,
                     int D, int omin, int omax, bool interp, int unary, float *out, cudaStream_t st,
                     int npairs = 1, long fps = 0);

// same on the tensor cores: BF16 features [2 * npairs][H][W][cp] (left
// images, then right), an integer disparity list (h_list on the host, d_list
// its device copy) cut into at most 4 parts whose bands are <= 128 wide (one
// part under the softmax unary); corr_tc_supported says whether a list
// qualifies.  err: the bounded-wait error flag.  outq (optional): the
// volume's 16-bit fixed-point copy (unary_q16), the BF16 path's CRF unary;
// out may then be null (no FP32 volume written).
bool corr_tc_supported(int C, int cp, const float *h_list, int D, int unary);
int correlation_tc(const void *feat, int npairs, int H, int W, int C, int cp, const float *d_list,
                   const float *h_list, int D, int unary, float *out, int *err, cudaStream_t st,
                   void *outq = nullptr);
// The BF16 path's 16-bit fixed-point unary: x = q * scale + offset (q in
// 0..65535), exact in FP32.  1 - <fL,fR> in [-2^-8, 2 - 2^-8] at 2^-15,
// -softmax in [-1, 0] at 2^-16.  false for a unary with no fixed range.
struct UnaryQ16 {
    float scale, offset;
};
bool unary_q16(int unary, UnaryQ16 *q);

// ------------------------------------------------------------ training step (k_train.cu)
// npz layout w[co][ci][kh][kw] -> conv_simt's wt [K][128] (if wt), the input
// gradient's wd [kh*kw*Cout][128] (if wd), bias padded to 128 (if b and b128)
int train_weight_layouts(const float *w, const float *b, int Cout, int Cin, int kh, int kw, float *wt, float *wd,
                         float *b128, cudaStream_t st);
// the BF16 mode's tensor-core weight layout [np][kh*kw][cp] and its |1x1| head
int train_w16(const float *w, int Cout, int Cin, int kh, int kw, int np, int cp, void *w16, cudaStream_t st);
// the input gradient's tensor-core layout [np][kh*kw][cp]: w16d[ci][tap][co] = w[co][ci][ky][kx], unflipped
int train_w16_dgrad(const float *w, int Cout, int Cin, int kh, int kw, int np, int cp, void *w16d, cudaStream_t st);
// zero the (p, q) border of BF16 [n][H + 2p][W + 2q][cp] (all channels)
int train_zero_border(void *buf, int nimg, int H, int W, int cp, int p, int q, cudaStream_t st);
// dy *= 1 - y^2 (y BF16) and a BF16 copy with a (p, q) zero border and channels padded to cp (conv_tc's input)
int train_tanh_bwd_pad(float *dy, const void *y, int nimg, int H, int W, int C, int ys, int p, int q, int cp,
                       void *out, cudaStream_t st);
int train_head2_bf16(const void *y2, int nimg, int npx, int P, int cs, const float *wh, float *out, cudaStream_t st);
// Activations y are FP32 or BF16 (bf16) at channel stride ys; gradients are dense FP32 [px][C].
int train_tanh_bwd(float *dy, const void *y, bool bf16, long npx, int C, int ys, cudaStream_t st); // dy *= 1 - y^2
int train_pad_zero(const float *in, int nimg, int H, int W, int C, int p, int q, float *out, cudaStream_t st);
int train_l2norm_bwd(const void *y, bool bf16, int ys, const float *df, long npx, int C, float *dy, cudaStream_t st);
// BF16 mode, the last feature layer: the L2 normalisation's adjoint times tanh' in one pass, written as BF16
// [n][H + 2p][W + 2q][128] inside a zeroed border; the per-channel sums in *nsplit rows (at most 4 x SMs) of part
int train_l2norm_tanh_bwd_pad(const void *y, int ys, const float *df, int nimg, int H, int W, int C, int p, int q,
                              void *out, float *part, int *nsplit, cudaStream_t st);
// one-minus-dot unary over an integer stored list (band [omin, omax]): dfl, dfr (dense) from dL/dvol;
// features at channel stride fs
int train_corr_bwd(const void *fl, const void *fr, bool bf16, int fs, const float *gvol, const float *d_list,
                   int npairs, int H, int W, int C, int D, int omin, int omax, float *dfl, float *dfr, cudaStream_t st);
// the same on the tensor cores (k_corr_bwd_tc.cu): BF16 features at channel stride fs (a multiple of
// 64); the list's offsets must be distinct.  err: the bounded-wait error flag
bool corr_bwd_tc_supported(int C, int fs, int D, int omin, int omax);
int corr_bwd_tc(const void *fl, const void *fr, int fs, const float *gvol, const float *d_list, int npairs, int H,
                int W, int C, int D, int omin, int omax, float *dfl, float *dfr, int *err, cudaStream_t st);
// pixel splits of the bias gradient's fixed-order reduction for P output pixels (about four per SM)
int train_wgrad_splits(long P);
// pixel splits of the weight gradient (K = kh*kw*Cin): about four CTAs per SM, >= 512 pixels each
int train_wgrad_splits_k(long P, int K);
// dw (npz layout) += weight gradient, db += bias gradient (if db); part:
// train_wgrad_splits_k x Cout x kh*kw*Cin floats, partb: train_wgrad_splits x Cout floats of scratch
int train_wgrad(const float *dz, int Cout, const void *in, bool bf16, long in_pix, long in_row, long in_img, int Cin,
                int kh, int kw, int nimg, int Ho, int Wo, float *part, float *dw, float *db, float *partb, cudaStream_t st);
int train_head_bwd(const void *y2, bool bf16, int ys, const float *wh, const float *gpw, int nimg, int npx, int P,
                   float *gh, float *dy2, cudaStream_t st);
// BF16 mode, P <= 64: the head's adjoint and the layer below's tanh' in one pass: gh (FP32 [px][2]) and dz as
// BF16 [n][H + 2p][W + 2q][64] inside a zeroed border; per-channel sums of dz in *nsplit rows of part
int train_head_tanh_bwd_pad(const void *y2, int ys, const float *wh, const float *gpw, int nimg, int H, int W, int P,
                            int p, int q, float *gh, void *out, float *part, int *nsplit, cudaStream_t st);
int train_bias_grad(const float *dz, int Cout, long P, float *partb, float *db, cudaStream_t st); // db += sum dz
int train_bias_reduce(const float *part, int nsplit, int Cout, float *db, cudaStream_t st); // db += sum of rows
// the 1x1 pairwise head (2 outputs): dw[o][c] += sum_p gh[p][o] y[p][c]; part: train_wgrad_splits(P) x 2C floats
int train_wgrad_head(const float *gh, const void *y, bool bf16, int ys, long P, int C, float *part, float *dw,
                     cudaStream_t st);
// BF16 copy of FP32 [npx][C] (C <= 64) at channel stride 64, zero padded
int train_to_bf16_c64(const float *in, long npx, int C, void *out, cudaStream_t st);
// the weight gradient on the tensor cores (k_wgrad_tc.cu), both operands NHWC BF16: dzpad = the output
// gradient with a (kh-1, kw-1) zero border, channel stride cpa (train_tanh_bwd_pad's copy); the layer
// input at the given element strides (pixel stride a multiple of 64).  dw (npz layout) += dW.
// scratch: wgrad_tc_scratch_bytes for wgrad_tc_splits(kh, nimg * Ho * ceil(Wo / 64)) splits;
// err: the bounded-wait error flag
bool wgrad_tc_supported(int Cout, int Cin, int kh, int kw);
int wgrad_tc_splits(int kh, long steps);
size_t wgrad_tc_scratch_bytes(int Cout, int Cin, int kh, int kw, int splits);
int wgrad_tc(const void *dzpad, int Cout, int cpa, const void *in, long in_pix, long in_row, long in_img, int Cin,
             int kh, int kw, int nimg, int Ho, int Wo, void *scratch, size_t scratch_bytes, float *dw, int *err,
             cudaStream_t st);
int train_augment(const float *vol, const int32_t *gt, long npx, int D, float *aug, int *err, cudaStream_t st);
int train_hinge(const float *vol, const float *w, const int32_t *gt, const int32_t *yh, int npairs, int W, int H,
                int D, float lam, const float rho[9], float L2, int delta, float gscale, float *gvol, float *gpw,
                double *contrib, double *rows, cudaStream_t st);
int train_sgd(float *theta, const float *g, float *v, long n, float lr, float mu, cudaStream_t st);

// ------------------------------------------------------------ census, edge weights, QuadDirect, LR check
constexpr int GAUSS_R = 3;           // Gaussian of the edge image: radius 3 >= 3 sigma
constexpr float GAUSS_SIGMA = 0.7f;  // stereo/stereo.cu:1092
int rgb_to_gray(const float *rgba, long n, float *gray, cudaStream_t st);
// d_list[z] = the z-th disparity (positive = left pixel x matches right x - d)
int census_volume(const float *g1, const float *g2, int W, int H, int fs, const float *d_list, int D, float lambda,
                  float *vol, cudaStream_t st);
void gauss_weights(float sigma, int R, float *w); // host: 2R+1 normalised weights
int edge_weights(const float *gray, int W, int H, float alpha, float beta, float lambda, float *tmp, float *tmp2,
                 const float *d_gw, float *wx, float *wy, cudaStream_t st);
int quadfit_direct(float *u, const float *c1, long npx, int D, float dmin, float dstep, cudaStream_t st);
int lr_check(const float *left, const float *right, int W, int H, float th, float *out, cudaStream_t st);

// ------------------------------------------------------------ CRF
struct CrfParams {
    float L1, L2;
    int delta;
    int shape;
    float slack;
};
// the solver's options as the C ABI passes them (ops slots L1, L2, delta,
// total_it of stereo/stereo.cpp:149-152): EUNSUPPORTED for a delta that is not
// an integer in 1..4, EINVAL for an unknown shape; shared by every entry point
// that takes a cnncrf_crf_options so all of them check in the same order
int crf_params(const cnncrf_crf_options *opt, CrfParams *p);
// workspace layout helpers
size_t crf_workspace_bytes(int W, int H, int D, int npairs = 1);
// npairs pairs at once: cost [n][H][W][D], weights [n][2][H][W] (wx, wy),
// labels [n][H][W]; bounds stay in the workspace (crf_lb_device).  keep_phi =
// false leaves the workspace's final phi unwritten (for callers that read the
// labels and bounds only, never C1).  costq (optional): the 16-bit
// fixed-point copy of cost (unary_q16) that the H passes read instead -- the
// BF16 path's unary; the solve is then the FP32 algorithm on the dequantised
// unary -- where D / 32 is even (crf_reads_q16).  With costq no pass reads
// cost (only the winner-take-all of iters <= 0 does).
int crf_solve_batch(const float *cost, const float *pw, int W, int H, int D, int npairs,
                    const CrfParams &p, int iters, int32_t *labels, void *ws, size_t ws_bytes,
                    cudaStream_t st, bool keep_phi = true, const void *costq = nullptr,
                    UnaryQ16 q = UnaryQ16{0.0f, 0.0f});
const double *crf_lb_device(const void *ws, int W, int H, int D, int npairs);
int crf_solve(const float *cost, const float *wx, const float *wy, int W, int H, int D,
              const CrfParams &p, int iters, int32_t *labels, void *ws, size_t ws_bytes,
              double *h_lb, cudaStream_t st, const void *costq = nullptr, UnaryQ16 q = UnaryQ16{0.0f, 0.0f});
// whether the H passes read a 16-bit cost copy at depth D (else they read the FP32 cost)
bool crf_reads_q16(int D);
// the slack_prop_2D_alg object of the C ABI reads costq instead of its cost when set
void slackprop_set_costq(struct ::cnncrf_slackprop *sp, const void *costq, UnaryQ16 q);
// theta - phi of the last solve (get_C1); costq: the 16-bit copy that solve read, if any
int crf_c1(const float *cost, const void *ws, long n, float *out, cudaStream_t st, int D = 0,
           const void *costq = nullptr, UnaryQ16 q = UnaryQ16{0.0f, 0.0f});

// CRF tile: prefetch ring depth (4 or 8 chain steps) and chains (warps) per
// CTA (1, 2 or 4) of the H and the V pass.  Every tile gives the same bits;
// only the speed differs.  The solver takes the tile of the process-wide
// tuning table for (W, H, D, npairs, delta), the default if there is none.
struct CrfTile {
    int ring_h = 8, wpb_h = 2, ring_v = 8, wpb_v = 2;
};
bool crf_tile_valid(const CrfTile &t);
CrfTile crf_tile_lookup(int W, int H, int D, int npairs, int delta);
void crf_tile_store(int W, int H, int D, int npairs, int delta, const CrfTile &t, float ms_h, float ms_v);
// time every tile on this problem (one H and one V pass each, best of 3)
// and, with store, enter the fastest per pass in the table; synchronises st
int crf_autotune(const float *cost, const float *wx, const float *wy, long wps, int W, int H, int D, int npairs,
                 const CrfParams &p, void *ws, size_t ws_bytes, cudaStream_t st, bool store = true,
                 const void *costq = nullptr, UnaryQ16 q = UnaryQ16{0.0f, 0.0f});

// ------------------------------------------------------------ small ops
int remap(float *out, const int32_t *labels, long n, float dmin, float dstep, cudaStream_t st);
int argmin(float *out, const float *vol, long npx, int D, float dmin, float dstep,
           cudaStream_t st);
int scale(float *x, long n, float s, cudaStream_t st);
int nchw_to_nhwc(const float *in, float *out, int C, long npx, cudaStream_t st);
// BF16 [npx][cs] -> FP32 [npx][C]
int bf16_to_f32(const void *in, int cs, int C, long npx, float *out, cudaStream_t st);
int warp_rgba(float *out, const float *in, const float *u, int W, int H, cudaStream_t st);
int tv_fit(const float *vol3, float *qf, int W, int H, float step, float lam, cudaStream_t st);
// TV/Huber primal-dual iterations, fused (k_tv.cu): from (u, p, q), or from
// (u, 0, 0) when pq_zero, `iters` iterations; the state ends in (u, p, q), the
// last iteration's u_ in u_.  ws >= tv_workspace_bytes(W, H), 256-byte aligned.
size_t tv_workspace_bytes(int W, int H);
int tv_iterate(float *u, float *u_, const float *u0, const float *qf, float *p, float *q,
               const float *wx, const float *wy, int W, int H, float C, float eps, float step,
               int iters, void *ws, size_t ws_bytes, bool pq_zero, cudaStream_t st);

// Bounded-wait self-test (k_selftest.cu): CNNCRF_ETIMEOUT when the probe's wait
// on a barrier that nothing completes (arrive == 0) gave up after `polls` polls.
int selftest_bounded_wait(int polls, int arrive, cudaStream_t st);

} // namespace k
} // namespace cnncrf
