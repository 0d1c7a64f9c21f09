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
// address.  The first call in each CUDA context (per device, and again after
// the device's primary context was reset) looks the real address up with
// cudaGetSymbolAddress, with that device current, and caches it under the
// context's unique id; that first call must come before any stream capture,
// and a first call made on a capturing stream is refused with ESTATE.
//
// All calls share the one array and it keeps whatever the last call left in
// it; the solver writes every scratch value before it reads it, so nothing
// has to start at zero.  Calls whose work overlaps on the GPU (different
// streams, or different host threads on the same device) race on the array
// and must be serialised by the caller.
#include <cuda.h>

#include <map>
#include <mutex>
#include <utility>

#include "common.h"
#include "kernels.h"

namespace {

constexpr size_t kStaticScratchBytes = 64ull << 20;

static __device__ __align__(256) unsigned char g_crf_scratch[kStaticScratchBytes];

std::mutex g_mu;
// (device, context id) -> address of g_crf_scratch in that context
std::map<std::pair<int, unsigned long long>, void *> g_addr;

// The unique id of the calling thread's current context (cuCtxGetId), through
// the runtime's driver entry points so the library needs no link to libcuda.
// 0 when the driver does not offer it: the address is then looked up on
// every call instead of cached.
unsigned long long current_context_id()
{
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q;
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (GetId)f;
        (void)cudaGetLastError();
    });
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

int scratch_address(cudaStream_t st, void **out)
{
    int dev = 0;
    CNNCRF_CUDA(cudaGetDevice(&dev));
    // a query that capture allows; it also makes the device's primary context
    // current on this thread, so the context id below is the one the solve runs in
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CNNCRF_CUDA(cudaStreamIsCapturing(st, &cs));
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lk(g_mu);
    if (ctx != 0) {
        auto it = g_addr.find({dev, ctx});
        if (it != g_addr.end()) {
            *out = it->second;
            return CNNCRF_OK;
        }
    }
    // the lookup may load this library's device code into the context, which
    // a stream capture does not allow
    if (cs != cudaStreamCaptureStatusNone)
        return cnncrf::fail(CNNCRF_ESTATE,
                            "crf_solve_static: the first call on device %d (and the first after a context reset) "
                            "must run outside stream capture: it looks up the scratch array's address",
                            dev);
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_crf_scratch);
    if (e != cudaSuccess || !p)
        return cnncrf::fail(CNNCRF_ECUDA, "crf_solve_static: cudaGetSymbolAddress failed on device %d: %s", dev,
                            cudaGetErrorString(e));
    if (ctx != 0) g_addr[{dev, ctx}] = p;
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
    // the options first, in cnncrf_crf_solve's order, then the sizes
    if (!opt) return fail(CNNCRF_EINVAL, "crf_solve_static: null options");
    k::CrfParams p;
    CNNCRF_TRY(k::crf_params(opt, &p));
    if (width < 1 || height < 1 || depth < 1)
        return fail(CNNCRF_EINVAL, "crf_solve_static: bad size %dx%dx%d", width, height, depth);
    const size_t need = k::crf_workspace_bytes(width, height, depth);
    if (need > kStaticScratchBytes)
        return fail(CNNCRF_EINVAL,
                    "crf_solve_static: a %dx%dx%d problem needs %zu bytes of scratch, the built-in array holds "
                    "%zu (64 MiB); use cnncrf_crf_solve with a caller workspace",
                    width, height, depth, need, kStaticScratchBytes);
    void *ws = nullptr;
    CNNCRF_TRY(scratch_address((cudaStream_t)stream, &ws));
    return k::crf_solve(d_cost, d_wx, d_wy, width, height, depth, p, opt->total_it, d_labels, ws,
                        kStaticScratchBytes, lower_bound, (cudaStream_t)stream);
}
