// crf_static.cu -- the CRF solve with no allocation at all, for callers that
// cannot call cudaMalloc.
//
// cnncrf_crf_solve needs a device workspace from its caller (two H x W x D
// float arrays plus the chain minima).  Some callers cannot allocate one: a
// plug-in hosted by a framework that owns every device allocation through its
// own pool and forbids direct cudaMalloc, or a real-time loop where a
// cudaMalloc / cudaFree -- which can stall the whole device -- would break
// the frame budget.  cnncrf_crf_solve_static runs the same solver with its
// workspace in a fixed array compiled into this library instead.
//
// The array: a file-scope `static __device__` buffer of 64 MiB.  Every GPU
// that loads the library holds it until the process exits.  It fits problems
// whose workspace (cnncrf_crf_workspace_size) is at most 64 MiB, roughly
// W x H x D <= 8 million labels; larger ones are rejected.
//
// On the host the name g_crf_scratch is only a stand-in, not a device
// address.  The first call on each device looks the real address up with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture.
//
// All calls share the one array and it keeps whatever the last call left in
// it; the solver writes every scratch value before it reads it, so nothing
// has to start at zero.  Calls whose work overlaps on the GPU (different
// streams, or different host threads on the same device) race on the array
// and must be serialised by the caller.
#include <map>
#include <mutex>

#include "common.h"
#include "kernels.h"

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;

static __device__ __align__(256) unsigned char g_crf_scratch[kStaticScratchBytes];

std::mutex g_mu;
std::map<int, void *> g_addr; // device -> address of g_crf_scratch on it

int scratch_address(void **out)
{
    int dev = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_addr.find(dev);
    if (it != g_addr.end()) {
        *out = it->second;
        return CNNCRF_OK;
    }
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_crf_scratch);
    if (e != cudaSuccess || !p)
        return cnncrf::fail(CNNCRF_ECUDA, "crf_solve_static: cudaGetSymbolAddress failed on device %d: %s", dev,
                            cudaGetErrorString(e));
    g_addr[dev] = p;
    *out = p;
    return CNNCRF_OK;
}

} // namespace

extern "C" int cnncrf_crf_solve_static(const float *d_cost, const float *d_wx, const float *d_wy, int width,
                                       int height, int depth, const cnncrf_crf_options *opt, int32_t *d_labels,
                                       double *lower_bound, cnncrf_stream_t stream)
{
    using namespace cnncrf;
    clear_error();
    if (!opt) return fail(CNNCRF_EINVAL, "crf_solve_static: null options");
    if (width < 1 || height < 1 || depth < 1)
        return fail(CNNCRF_EINVAL, "crf_solve_static: bad size %dx%dx%d", width, height, depth);
    const size_t need = k::crf_workspace_bytes(width, height, depth);
    if (need > kStaticScratchBytes)
        return fail(CNNCRF_EINVAL,
                    "crf_solve_static: a %dx%dx%d problem needs %zu bytes of scratch, the built-in array holds "
                    "%zu (64 MiB); use cnncrf_crf_solve with a caller workspace",
                    width, height, depth, need, kStaticScratchBytes);
    int delta = (int)opt->delta;
    if ((float)delta != opt->delta || delta < 1 || delta > 4)
        return fail(CNNCRF_EUNSUPPORTED, "crf_solve_static: delta %g must be an integer in 1..4", opt->delta);
    if (opt->shape != CNNCRF_RHO_STEP && opt->shape != CNNCRF_RHO_LINEAR)
        return fail(CNNCRF_EINVAL, "crf_solve_static: shape %d", opt->shape);
    k::CrfParams p;
    p.L1 = opt->L1;
    p.L2 = opt->L2;
    p.delta = delta;
    p.shape = opt->shape;
    p.slack = opt->slack;
    void *ws = nullptr;
    CNNCRF_TRY(scratch_address(&ws));
    return k::crf_solve(d_cost, d_wx, d_wy, width, height, depth, p, opt->total_it, d_labels, ws,
                        kStaticScratchBytes, lower_bound, (cudaStream_t)stream);
}
