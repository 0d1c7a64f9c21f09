// batch.cpp -- the batched form of Stereo::computeSlackPropagation for many
// pairs at once (cnncrf_batch_*; no counterpart in the reference, whose
// Stereo object holds one pair).
//
// Pairs with the same size and disparity range form a group (at most
// group_cap pairs each when a cap is set).  A group runs as one batch: one
// net over all its images (the tensor-core convolutions see 2n images per
// launch), one correlation launch, one CRF launch per pass over all n x H row
// chains / n x W column chains.
//
// The groups form a pipeline: the CNN part of a group (padding, both nets,
// correlation) runs on a high-priority stream after the CNN part of the
// previous group, and its CRF on a low-priority stream of its own.  The CNN
// kernels are bound by the tensor cores, the CRF by HBM, and a CRF CTA fits
// on an SM beside a convolution CTA, so the CNN of group i+1 runs while the
// CRF of group i streams its volume.  Everything is forked from and joined
// back into the batch's stream; with graph capture on, the whole sequence is
// captured once into a CUDA graph (node priorities kept) and replayed by
// later runs with the same parameters.
//
// cnncrf_batch_run_host takes the pairs' images in host memory and returns
// the disparities to host memory as part of the same pipeline: a copy stream
// carries every group's host-to-device copies ahead of that group's CNN, so
// group i+1's images travel while group i computes, and each group's
// disparities are copied back on its CRF stream right after its remap.
#include <cmath>
#include <memory>
#include <string>
#include <vector>

#include "common.h"
#include "kernels.h"
#include "net.h"

using namespace cnncrf;

namespace {

struct Group {
    int W = 0, H = 0, depth = 0;
    float dmin = 0, dstep = 1, dmax = 0;
    std::vector<int> members; // global pair indices, in batch order
    DevBuf img[2], padded[2], vol, volq, pw, out, labels, ws;
    cnncrf_net_t net = nullptr;
    cudaStream_t stream = nullptr;     // CNN part (high priority)
    cudaStream_t crf_stream = nullptr; // CRF part (low priority)
    cudaEvent_t cnn_done = nullptr, done = nullptr, in_done = nullptr;
    size_t ws_bytes = 0;
    bool vol_written = true; // the FP32 volume holds the last run's costs (else only volq does)
    ~Group()
    {
        if (net) cnncrf_net_destroy(net);
        if (in_done) cudaEventDestroy(in_done);
        if (done) cudaEventDestroy(done);
        if (cnn_done) cudaEventDestroy(cnn_done);
        if (stream) cudaStreamDestroy(stream);
        if (crf_stream) cudaStreamDestroy(crf_stream);
    }
};

int log2i(int num)
{
    int r = 0;
    while (num >>= 1) ++r;
    return r;
}

} // namespace

struct cnncrf_batch {
    cnncrf_stereo_options o{};
    int matching = CNNCRF_MATCH_COLORCNN_PAIRWISE, num_layers = 7, with_xy = 0;
    std::string param_base;
    bool xavier = true;
    uint64_t seed = 0;
    cudaStream_t st = nullptr;   // the caller's stream
    cudaStream_t work = nullptr; // the batch's own stream (capturable even when `st` is the legacy stream)
    cudaStream_t copy = nullptr; // host-to-device copies of run_host, ahead of the groups' CNN parts
    cudaEvent_t in_ev = nullptr, out_ev = nullptr;
    std::vector<std::unique_ptr<Group>> groups;
    std::vector<std::pair<int, int>> loc; // pair -> (group, slot)
    int group_cap = 0;                    // most pairs per group (0: no cap)
    bool keep_volume = false;             // BF16: also write the FP32 volume (cnncrf_batch_keep_volume)
    bool built = false;
    // graphs: one per (parameters, run_host buffers) key, the most recent
    // last; a key runs eagerly once (which also sets every kernel
    // attribute), is captured by its second run and replayed after that
    struct GraphEntry {
        float L1, L2, delta, lambda;
        int iters;
        std::vector<const void *> ptrs; // host buffers baked into the copy nodes (empty: run)
        cudaGraphExec_t exec;
    };
    static constexpr size_t kMaxGraphs = 4;
    bool use_graph = false;
    std::vector<GraphEntry> graphs;
    cudaEvent_t fork = nullptr;

    // host buffers of the current run_host call (null: images staged by set_images, no copy out)
    const float *const *h_left = nullptr, *const *h_right = nullptr;
    float *const *h_out = nullptr;

    ~cnncrf_batch()
    {
        invalidate();
        if (fork) cudaEventDestroy(fork);
        if (in_ev) cudaEventDestroy(in_ev);
        if (out_ev) cudaEventDestroy(out_ev);
        groups.clear();
        if (work) cudaStreamDestroy(work);
        if (copy) cudaStreamDestroy(copy);
    }
    void invalidate()
    {
        for (auto &g : graphs)
            if (g.exec) cudaGraphExecDestroy(g.exec);
        graphs.clear();
    }
    int build();
    int enqueue(float L1, float L2, float delta, int iters, float lambda);
    int run(float L1, float L2, float delta, int iterations, float lambda);
};

int cnncrf_batch::build()
{
    if (matching != CNNCRF_MATCH_COLORCNN_PAIRWISE && matching != CNNCRF_MATCH_GRAYCNN_PAIRWISE &&
        matching != CNNCRF_MATCH_CONCATCNN_PAIRWISE)
        return fail(CNNCRF_EUNSUPPORTED, "batch: only the pairwise matchings (COLORPAIR) are batched");
    bool gray = matching == CNNCRF_MATCH_GRAYCNN_PAIRWISE;
    const bool concat = matching == CNNCRF_MATCH_CONCATCNN_PAIRWISE; // FP32 only
    for (auto &gp : groups) {
        Group &g = *gp;
        const int n = (int)g.members.size();
        const size_t N = (size_t)g.W * g.H;
        cnncrf_net_desc d{};
        d.num_layers = num_layers;
        d.topology = concat ? CNNCRF_TOPO_CONCAT : o.topology;
        d.in_channels = gray ? 1 : (with_xy ? 5 : 3);
        d.feat_channels = concat ? 0 : o.feat_channels;
        d.unary = o.unary;
        d.precision = o.precision;
        d.with_pairwise = 1;
        d.pw_channels = o.pw_channels;
        const int pad = net_padding(d);
        if (g.net) cnncrf_net_destroy(g.net);
        g.net = nullptr;
        CNNCRF_TRY(cnncrf_net_create(&g.net, &d, n, g.H + 2 * pad, g.W + 2 * pad));
        int prio_low = 0, prio_high = 0;
        CNNCRF_CUDA(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
        if (!g.stream) CNNCRF_CUDA(cudaStreamCreateWithPriority(&g.stream, cudaStreamNonBlocking, prio_high));
        if (!g.crf_stream) CNNCRF_CUDA(cudaStreamCreateWithPriority(&g.crf_stream, cudaStreamNonBlocking, prio_low));
        if (!g.done) CNNCRF_CUDA(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
        if (!g.cnn_done) CNNCRF_CUDA(cudaEventCreateWithFlags(&g.cnn_done, cudaEventDisableTiming));
        if (!g.in_done) CNNCRF_CUDA(cudaEventCreateWithFlags(&g.in_done, cudaEventDisableTiming));
        CNNCRF_TRY(cnncrf_net_set_stream(g.net, (cnncrf_stream_t)g.stream));
        for (int s = 0; s < 2; ++s) {
            CNNCRF_TRY(g.img[s].reserve(sizeof(float) * 4 * N * n));
            CNNCRF_TRY(g.padded[s].reserve(sizeof(float) * 4 * (size_t)(g.W + 2 * pad) * (g.H + 2 * pad) * n));
        }
        CNNCRF_TRY(g.vol.reserve(sizeof(float) * N * g.depth * n));
        // the BF16 path's CRF reads the volume's 16-bit fixed-point copy, which the correlation writes instead
        // of the FP32 volume (no caller of the batch reads that; the CRF's winner-take-all at 0 iterations does)
        k::UnaryQ16 uq;
        if (o.precision == CNNCRF_BF16 && k::crf_reads_q16(g.depth) && k::unary_q16(o.unary, &uq))
            CNNCRF_TRY(g.volq.reserve(2 * N * g.depth * n));
        CNNCRF_TRY(g.pw.reserve(sizeof(float) * 2 * N * n));
        CNNCRF_TRY(g.out.reserve(sizeof(float) * N * n));
        CNNCRF_TRY(g.labels.reserve(sizeof(int32_t) * N * n));
        g.ws_bytes = k::crf_workspace_bytes(g.W, g.H, g.depth, n);
        CNNCRF_TRY(g.ws.reserve(g.ws_bytes));
        CNNCRF_TRY(cnncrf_net_init(g.net, g.dmin, g.dmax, g.dstep, 0, g.vol.as<float>(), g.pw.as<float>()));
        g.net->volq = g.volq.get();
        if (g.net->D != g.depth)
            return fail(CNNCRF_ESHAPE, "batch: disparity list has %d entries, volume depth %d", g.net->D, g.depth);
        if (xavier) CNNCRF_TRY(cnncrf_net_init_xavier(g.net, seed));
        else CNNCRF_TRY(cnncrf_net_set_all_params(g.net, (param_base + ".npz").c_str()));
    }
    if (!fork) CNNCRF_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    if (!in_ev) CNNCRF_CUDA(cudaEventCreateWithFlags(&in_ev, cudaEventDisableTiming));
    if (!out_ev) CNNCRF_CUDA(cudaEventCreateWithFlags(&out_ev, cudaEventDisableTiming));
    if (!work) CNNCRF_CUDA(cudaStreamCreateWithFlags(&work, cudaStreamNonBlocking));
    if (!copy) CNNCRF_CUDA(cudaStreamCreateWithFlags(&copy, cudaStreamNonBlocking));
    CNNCRF_CUDA(cudaDeviceSynchronize()); // parameter uploads done before any stream work
    built = true;
    return CNNCRF_OK;
}

// fork -> the groups' CNN parts one after another, each group's CRF after
// its CNN -> join, all enqueued from `work`
int cnncrf_batch::enqueue(float L1, float L2, float delta, int iters, float lambda)
{
    k::CrfParams p;
    int di = (int)delta;
    if ((float)di != delta || di < 1 || di > 4) return fail(CNNCRF_EUNSUPPORTED, "batch: delta %g", delta);
    p.L1 = L1, p.L2 = L2, p.delta = di, p.shape = o.crf_shape, p.slack = o.crf_slack;
    k::UnaryQ16 uq{1.0f, 0.0f};
    k::unary_q16(o.unary, &uq);
    CNNCRF_CUDA(cudaEventRecord(fork, work));
    if (h_left) CNNCRF_CUDA(cudaStreamWaitEvent(copy, fork, 0));
    cudaEvent_t prev = fork;
    for (auto &gp : groups) {
        Group &g = *gp;
        const int n = (int)g.members.size();
        const long N = (long)g.W * g.H;
        cudaStream_t gs = g.stream, cs = g.crf_stream;
        CNNCRF_CUDA(cudaStreamWaitEvent(gs, prev, 0));
        if (h_left) { // this group's images, on the copy stream in pipeline order
            const size_t bytes = sizeof(float) * 4 * (size_t)N;
            for (int m = 0; m < n; ++m) {
                const int pair = g.members[m];
                CNNCRF_CUDA(cudaMemcpyAsync((char *)g.img[0].get() + bytes * m, h_left[pair], bytes,
                                            cudaMemcpyHostToDevice, copy));
                CNNCRF_CUDA(cudaMemcpyAsync((char *)g.img[1].get() + bytes * m, h_right[pair], bytes,
                                            cudaMemcpyHostToDevice, copy));
            }
            CNNCRF_CUDA(cudaEventRecord(g.in_done, copy));
            CNNCRF_CUDA(cudaStreamWaitEvent(gs, g.in_done, 0));
        }
        const int pad = g.net->pad;
        CNNCRF_TRY(k::pad_rgba(g.img[0].as<float>(), g.W, g.H, pad, g.padded[0].as<float>(), gs, n));
        CNNCRF_TRY(k::pad_rgba(g.img[1].as<float>(), g.W, g.H, pad, g.padded[1].as<float>(), gs, n));
        g.net->vol_fp32 = keep_volume || iters <= 0;
        CNNCRF_TRY(g.net->predict(g.padded[0].as<float>(), g.padded[1].as<float>()));
        g.vol_written = !(g.net->volq_valid && !g.net->vol_fp32);
        CNNCRF_TRY(k::scale(g.pw.as<float>(), 2 * N * n, lambda, gs)); // stereo/stereo.cpp:136-137
        CNNCRF_CUDA(cudaEventRecord(g.cnn_done, gs));
        prev = g.cnn_done;
        CNNCRF_CUDA(cudaStreamWaitEvent(cs, g.cnn_done, 0));
        CNNCRF_TRY(k::crf_solve_batch(g.vol.as<float>(), g.pw.as<float>(), g.W, g.H, g.depth, n, p, iters,
                                      g.labels.as<int32_t>(), g.ws.get(), g.ws_bytes, cs,
                                      false, // labels and bounds only: the last phi is dead
                                      g.net->volq_valid ? g.volq.get() : nullptr, uq));
        CNNCRF_TRY(k::remap(g.out.as<float>(), g.labels.as<int32_t>(), N * n, g.dmin, g.dstep, cs));
        if (h_out)
            for (int m = 0; m < n; ++m)
                if (h_out[g.members[m]])
                    CNNCRF_CUDA(cudaMemcpyAsync(h_out[g.members[m]], g.out.as<float>() + N * m,
                                                sizeof(float) * N, cudaMemcpyDeviceToHost, cs));
        CNNCRF_CUDA(cudaEventRecord(g.done, cs));
        CNNCRF_CUDA(cudaStreamWaitEvent(work, g.done, 0));
    }
    return CNNCRF_OK;
}

extern "C" {

int cnncrf_batch_create(cnncrf_batch_t *b, const cnncrf_stereo_options *opt)
{
    clear_error();
    if (!b) return fail(CNNCRF_EINVAL, "null argument");
    auto *bt = new cnncrf_batch;
    if (opt) bt->o = *opt;
    else cnncrf_stereo_default_options(&bt->o);
    *b = bt;
    return CNNCRF_OK;
}

int cnncrf_batch_destroy(cnncrf_batch_t b)
{
    if (b) cudaDeviceSynchronize();
    delete b;
    return CNNCRF_OK;
}

int cnncrf_batch_set_stream(cnncrf_batch_t b, cnncrf_stream_t stream)
{
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    b->st = (cudaStream_t)stream;
    b->invalidate();
    return CNNCRF_OK;
}

int cnncrf_batch_set_network(cnncrf_batch_t b, int matching, int num_layers, int with_xy, const char *param_base,
                             uint64_t seed)
{
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    b->matching = matching;
    b->num_layers = num_layers;
    b->with_xy = with_xy ? 1 : 0;
    b->xavier = param_base == nullptr;
    if (param_base) b->param_base = param_base;
    b->seed = seed;
    b->built = false;
    b->invalidate();
    return CNNCRF_OK;
}

int cnncrf_batch_add_pair(cnncrf_batch_t b, int width, int height, float disp_min, float disp_step, float disp_max,
                          int *pair_index)
{
    clear_error();
    if (!b || !pair_index) return fail(CNNCRF_EINVAL, "null argument");
    if (width < 1 || height < 1 || !(disp_step > 0.0f)) return fail(CNNCRF_EINVAL, "add_pair: bad size / step");
    int depth = (int)((disp_max - disp_min) / disp_step + 1);
    if (depth < 1) return fail(CNNCRF_EINVAL, "add_pair: empty disparity range");
    if (b->o.ref_depth_rounding) depth = std::min(256, 1 << (log2i(depth - 1) + 1));
    float dmax = disp_min + (depth - 1) * disp_step;
    int gi = -1;
    for (size_t i = 0; i < b->groups.size(); ++i) {
        Group &g = *b->groups[i];
        if (g.W == width && g.H == height && g.dmin == disp_min && g.dstep == disp_step && g.depth == depth &&
            (b->group_cap <= 0 || (int)g.members.size() < b->group_cap)) {
            gi = (int)i;
            break;
        }
    }
    if (gi < 0) {
        b->groups.emplace_back(new Group);
        Group &g = *b->groups.back();
        g.W = width, g.H = height, g.depth = depth, g.dmin = disp_min, g.dstep = disp_step, g.dmax = dmax;
        gi = (int)b->groups.size() - 1;
    }
    Group &g = *b->groups[gi];
    *pair_index = (int)b->loc.size();
    b->loc.push_back({gi, (int)g.members.size()});
    g.members.push_back(*pair_index);
    b->built = false;
    b->invalidate();
    return CNNCRF_OK;
}

int cnncrf_batch_set_group_size(cnncrf_batch_t b, int max_pairs)
{
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    if (max_pairs < 0) return fail(CNNCRF_EINVAL, "set_group_size: %d", max_pairs);
    if (!b->loc.empty()) return fail(CNNCRF_ESTATE, "set_group_size: call it before the first add_pair");
    b->group_cap = max_pairs;
    return CNNCRF_OK;
}

int cnncrf_batch_keep_volume(cnncrf_batch_t b, int enable)
{
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    b->keep_volume = enable != 0;
    b->invalidate(); // the captured correlations write one volume or the other
    return CNNCRF_OK;
}

int cnncrf_batch_num_pairs(cnncrf_batch_t b, int *n)
{
    if (!b || !n) return fail(CNNCRF_EINVAL, "null argument");
    *n = (int)b->loc.size();
    return CNNCRF_OK;
}

static int stage(cnncrf_batch_t b, int pair, const float *l, const float *r, cudaMemcpyKind kind)
{
    if (!b || !l || !r) return fail(CNNCRF_EINVAL, "set_images: null argument");
    if (pair < 0 || pair >= (int)b->loc.size()) return fail(CNNCRF_EINVAL, "set_images: pair %d", pair);
    if (!b->built) CNNCRF_TRY(b->build());
    Group &g = *b->groups[b->loc[pair].first];
    const size_t bytes = sizeof(float) * 4 * (size_t)g.W * g.H;
    const size_t off = bytes * b->loc[pair].second;
    CNNCRF_CUDA(cudaMemcpyAsync((char *)g.img[0].get() + off, l, bytes, kind, b->st));
    CNNCRF_CUDA(cudaMemcpyAsync((char *)g.img[1].get() + off, r, bytes, kind, b->st));
    return CNNCRF_OK;
}

int cnncrf_batch_set_images(cnncrf_batch_t b, int pair, const float *h_left, const float *h_right)
{
    clear_error();
    return stage(b, pair, h_left, h_right, cudaMemcpyHostToDevice);
}

int cnncrf_batch_set_images_device(cnncrf_batch_t b, int pair, const float *d_left, const float *d_right)
{
    clear_error();
    return stage(b, pair, d_left, d_right, cudaMemcpyDeviceToDevice);
}

int cnncrf_batch_use_graph(cnncrf_batch_t b, int enable)
{
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    b->use_graph = enable != 0;
    b->invalidate();
    return CNNCRF_OK;
}

int cnncrf_batch_autotune(cnncrf_batch_t b, float L1, float L2, float delta, int iterations, float lambda_reg)
{
    clear_error();
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    CNNCRF_TRY(cnncrf_batch_run(b, L1, L2, delta, iterations, lambda_reg)); // every group's volume and weights
    CNNCRF_CUDA(cudaStreamSynchronize(b->st));
    CNNCRF_TRY(cnncrf_batch_check(b));
    k::CrfParams p;
    p.L1 = L1, p.L2 = L2, p.delta = (int)delta, p.shape = b->o.crf_shape, p.slack = b->o.crf_slack;
    k::UnaryQ16 uq{1.0f, 0.0f};
    k::unary_q16(b->o.unary, &uq);
    for (auto &gp : b->groups) {
        Group &g = *gp;
        const long N = (long)g.W * g.H;
        CNNCRF_TRY(k::crf_autotune(g.vol.as<float>(), g.pw.as<float>(), g.pw.as<float>() + N, 2 * N, g.W, g.H,
                                   g.depth, (int)g.members.size(), p, g.ws.get(), g.ws_bytes, b->work, true,
                                   g.net->volq_valid ? g.volq.get() : nullptr, uq));
    }
    // the tensor-core convolutions' launch forms, per layer shape of every group's net
    for (auto &gp : b->groups) CNNCRF_TRY(gp->net->autotune_conv());
    b->invalidate(); // the captured launches carry the old tiles and forms
    return CNNCRF_OK;
}

int cnncrf_batch_num_groups(cnncrf_batch_t b, int *n)
{
    if (!b || !n) return fail(CNNCRF_EINVAL, "null argument");
    *n = (int)b->groups.size();
    return CNNCRF_OK;
}

int cnncrf_batch_group_shape(cnncrf_batch_t b, int group, int *width, int *height, int *depth, int *npairs)
{
    if (!b || !width || !height || !depth || !npairs) return fail(CNNCRF_EINVAL, "null argument");
    if (group < 0 || group >= (int)b->groups.size()) return fail(CNNCRF_EINVAL, "group %d", group);
    const Group &g = *b->groups[group];
    *width = g.W, *height = g.H, *depth = g.depth, *npairs = (int)g.members.size();
    return CNNCRF_OK;
}

// one run of the whole batch from the caller's stream; with graphs on, the
// first run of a (parameters, run_host buffers) key is eager, the next one
// captures it, later ones replay its graph
int cnncrf_batch::run(float L1, float L2, float delta, int iterations, float lambda_reg)
{
    if (loc.empty()) return fail(CNNCRF_ESTATE, "batch: no pairs");
    if (!built) CNNCRF_TRY(build());
    // the host buffers of run_host go into the graph's copy nodes: a graph
    // replays only with the same buffers, and only page-locked ones can be
    // captured (pageable buffers run eagerly)
    std::vector<const void *> ptrs;
    bool capturable = true;
    if (h_left) {
        for (size_t i = 0; i < loc.size(); ++i) {
            const void *pp[3] = {h_left[i], h_right[i], h_out ? h_out[i] : nullptr};
            for (const void *q : pp) {
                ptrs.push_back(q);
                if (!q) continue;
                cudaPointerAttributes at{};
                if (cudaPointerGetAttributes(&at, q) != cudaSuccess || at.type != cudaMemoryTypeHost) {
                    (void)cudaGetLastError();
                    capturable = false;
                }
            }
        }
    }
    // hand over from the caller's stream (image copies) to the batch's stream
    CNNCRF_CUDA(cudaEventRecord(in_ev, st));
    CNNCRF_CUDA(cudaStreamWaitEvent(work, in_ev, 0));
    int rc = CNNCRF_OK;
    GraphEntry *ge = nullptr;
    for (auto &g : graphs)
        if (g.iters == iterations && g.L1 == L1 && g.L2 == L2 && g.delta == delta && g.lambda == lambda_reg &&
            g.ptrs == ptrs)
            ge = &g;
    if (!use_graph || !capturable) {
        rc = enqueue(L1, L2, delta, iterations, lambda_reg);
    } else if (ge && ge->exec) {
        cudaError_t e = cudaGraphLaunch(ge->exec, work);
        if (e != cudaSuccess) rc = fail(CNNCRF_ECUDA, "batch: graph launch: %s", cudaGetErrorString(e));
    } else if (!ge) { // first run of this key: eager
        rc = enqueue(L1, L2, delta, iterations, lambda_reg);
        if (rc == CNNCRF_OK) {
            if (graphs.size() >= kMaxGraphs) {
                if (graphs.front().exec) cudaGraphExecDestroy(graphs.front().exec);
                graphs.erase(graphs.begin());
            }
            graphs.push_back(GraphEntry{L1, L2, delta, lambda_reg, iterations, ptrs, nullptr});
        }
    } else { // second run: capture, then launch
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(work, cudaStreamCaptureModeRelaxed);
        if (e != cudaSuccess) {
            rc = fail(CNNCRF_ECUDA, "batch: begin capture: %s", cudaGetErrorString(e));
        } else {
            rc = enqueue(L1, L2, delta, iterations, lambda_reg);
            e = cudaStreamEndCapture(work, &g);
            if (rc == CNNCRF_OK && e != cudaSuccess)
                rc = fail(CNNCRF_ECUDA, "batch: graph capture failed: %s", cudaGetErrorString(e));
            if (rc == CNNCRF_OK) {
                e = cudaGraphInstantiateWithFlags(&ge->exec, g, cudaGraphInstantiateFlagUseNodePriority);
                if (e != cudaSuccess) {
                    ge->exec = nullptr;
                    rc = fail(CNNCRF_ECUDA, "batch: graph instantiation failed: %s", cudaGetErrorString(e));
                }
            }
            if (g) cudaGraphDestroy(g);
            if (rc == CNNCRF_OK) {
                e = cudaGraphLaunch(ge->exec, work);
                if (e != cudaSuccess) rc = fail(CNNCRF_ECUDA, "batch: graph launch: %s", cudaGetErrorString(e));
            }
        }
    }
    // hand back: the caller's stream sees the results after this point
    CNNCRF_CUDA(cudaEventRecord(out_ev, work));
    CNNCRF_CUDA(cudaStreamWaitEvent(st, out_ev, 0));
    return rc;
}

int cnncrf_batch_run(cnncrf_batch_t b, float L1, float L2, float delta, int iterations, float lambda_reg)
{
    CNNCRF_RANGE("batch_run");
    clear_error();
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    b->h_left = b->h_right = nullptr;
    b->h_out = nullptr;
    return b->run(L1, L2, delta, iterations, lambda_reg);
}

int cnncrf_batch_run_host(cnncrf_batch_t b, const float *const *h_left, const float *const *h_right,
                          float *const *h_out, float L1, float L2, float delta, int iterations, float lambda_reg)
{
    CNNCRF_RANGE("batch_run_host");
    clear_error();
    if (!b || !h_left || !h_right) return fail(CNNCRF_EINVAL, "run_host: null argument");
    for (size_t i = 0; i < b->loc.size(); ++i)
        if (!h_left[i] || !h_right[i]) return fail(CNNCRF_EINVAL, "run_host: null image of pair %zu", i);
    b->h_left = h_left, b->h_right = h_right, b->h_out = h_out;
    const int rc = b->run(L1, L2, delta, iterations, lambda_reg);
    b->h_left = b->h_right = nullptr;
    b->h_out = nullptr;
    return rc;
}

static Group *group_of(cnncrf_batch_t b, int pair, size_t *off_px)
{
    if (!b || pair < 0 || pair >= (int)b->loc.size() || !b->built) return nullptr;
    Group *g = b->groups[b->loc[pair].first].get();
    *off_px = (size_t)g->W * g->H * b->loc[pair].second;
    return g;
}

int cnncrf_batch_get_output(cnncrf_batch_t b, int pair, float *h_out)
{
    size_t off;
    Group *g = group_of(b, pair, &off);
    if (!g || !h_out) return fail(CNNCRF_EINVAL, "get_output: bad pair / null output");
    CNNCRF_CUDA(cudaMemcpyAsync(h_out, g->out.as<float>() + off, sizeof(float) * g->W * g->H,
                                cudaMemcpyDeviceToHost, b->st));
    CNNCRF_CUDA(cudaStreamSynchronize(b->st));
    return CNNCRF_OK;
}

int cnncrf_batch_get_output_device(cnncrf_batch_t b, int pair, const float **d_out)
{
    size_t off;
    Group *g = group_of(b, pair, &off);
    if (!g || !d_out) return fail(CNNCRF_EINVAL, "get_output_device: bad pair");
    *d_out = g->out.as<float>() + off;
    return CNNCRF_OK;
}

int cnncrf_batch_get_labels_device(cnncrf_batch_t b, int pair, const int32_t **d_labels)
{
    size_t off;
    Group *g = group_of(b, pair, &off);
    if (!g || !d_labels) return fail(CNNCRF_EINVAL, "get_labels_device: bad pair");
    *d_labels = g->labels.as<int32_t>() + off;
    return CNNCRF_OK;
}

int cnncrf_batch_get_volume_device(cnncrf_batch_t b, int pair, const float **d_vol, int *depth)
{
    size_t off;
    Group *g = group_of(b, pair, &off);
    if (!g || !d_vol) return fail(CNNCRF_EINVAL, "get_volume_device: bad pair");
    if (!g->vol_written)
        return fail(CNNCRF_ESTATE, "get_volume_device: the BF16 batch kept only the CRF's 16-bit copy of the "
                                   "volume; call cnncrf_batch_keep_volume(b, 1) before the run");
    *d_vol = g->vol.as<float>() + off * g->depth;
    if (depth) *depth = g->depth;
    return CNNCRF_OK;
}

int cnncrf_batch_lower_bound(cnncrf_batch_t b, int pair, double *lb)
{
    size_t off;
    Group *g = group_of(b, pair, &off);
    if (!g || !lb) return fail(CNNCRF_EINVAL, "lower_bound: bad pair");
    const double *d = k::crf_lb_device(g->ws.get(), g->W, g->H, g->depth, (int)g->members.size());
    CNNCRF_CUDA(cudaMemcpyAsync(lb, d + b->loc[pair].second, sizeof(double), cudaMemcpyDeviceToHost, b->st));
    CNNCRF_CUDA(cudaStreamSynchronize(b->st));
    return CNNCRF_OK;
}

int cnncrf_batch_check(cnncrf_batch_t b)
{
    if (!b) return fail(CNNCRF_EINVAL, "null batch");
    CNNCRF_CUDA(cudaStreamSynchronize(b->st));
    for (auto &g : b->groups)
        if (g->net) CNNCRF_TRY(g->net->check_error());
    return CNNCRF_OK;
}

} // extern "C"
