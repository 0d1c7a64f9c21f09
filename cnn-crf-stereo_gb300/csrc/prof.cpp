// prof.cpp -- launch counter, NVTX ranges and optional per-kernel CUDA-event
// timing behind cnncrf_kernel_launches / cnncrf_profile_* (instrumentation;
// no counterpart in the reference, whose only timer was iu::IuCudaTimer
// around whole stages, stereo/stereonet.cpp:258-315).  NVTX is the CUDA
// toolkit's header-only NVTX 3: without an attached tool each range is one
// check of an unset function pointer.
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.h"

namespace cnncrf {

namespace {
std::atomic<uint64_t> g_launches{0};
std::atomic<bool> g_enabled{false};
std::mutex g_mu;
struct Rec {
    cudaEvent_t a, b;
};
std::map<std::string, std::vector<Rec>> g_recs;
std::vector<cudaEvent_t> g_pool;

nvtxDomainHandle_t domain()
{
    static nvtxDomainHandle_t d = nvtxDomainCreateA("cnncrf");
    return d;
}

void range_push(const char *name)
{
    nvtxEventAttributes_t a = {};
    a.version = NVTX_VERSION;
    a.size = NVTX_EVENT_ATTRIB_STRUCT_SIZE;
    a.messageType = NVTX_MESSAGE_TYPE_ASCII;
    a.message.ascii = name;
    nvtxDomainRangePushEx(domain(), &a);
}

cudaEvent_t get_event()
{
    if (!g_pool.empty()) {
        cudaEvent_t e = g_pool.back();
        g_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}
} // namespace

Range::Range(const char *name) { range_push(name); }
Range::~Range() { nvtxDomainRangePop(domain()); }

Prof::Prof(const char *name, cudaStream_t st) : name_(name), st_(st)
{
    range_push(name);
    if (g_enabled.load(std::memory_order_relaxed)) {
        std::lock_guard<std::mutex> lk(g_mu);
        a_ = get_event();
        if (a_) cudaEventRecord(a_, st_);
    }
}

Prof::~Prof()
{
    nvtxDomainRangePop(domain());
    g_launches.fetch_add(1, std::memory_order_relaxed);
    if (a_) {
        std::lock_guard<std::mutex> lk(g_mu);
        cudaEvent_t b = get_event();
        if (b) {
            cudaEventRecord(b, st_);
            g_recs[name_].push_back({a_, b});
        } else {
            g_pool.push_back(a_);
        }
    }
}

} // namespace cnncrf

using namespace cnncrf;

extern "C" {

int cnncrf_kernel_launches(uint64_t *count)
{
    if (!count) return fail(CNNCRF_EINVAL, "null argument");
    *count = g_launches.load();
    return CNNCRF_OK;
}

int cnncrf_profile_enable(int enable)
{
    g_enabled.store(enable != 0);
    return CNNCRF_OK;
}

int cnncrf_profile_reset(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto &kv : g_recs)
        for (auto &r : kv.second) {
            cudaEventSynchronize(r.b);
            g_pool.push_back(r.a);
            g_pool.push_back(r.b);
        }
    g_recs.clear();
    return CNNCRF_OK;
}

int cnncrf_profile_query(const char *kernel, int *launches, double *total_ms)
{
    if (!kernel || !launches || !total_ms) return fail(CNNCRF_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(g_mu);
    *launches = 0;
    *total_ms = 0.0;
    auto it = g_recs.find(kernel);
    if (it == g_recs.end()) return CNNCRF_OK;
    for (auto &r : it->second) {
        CNNCRF_CUDA(cudaEventSynchronize(r.b));
        float ms = 0.0f;
        CNNCRF_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        *total_ms += ms;
        ++*launches;
    }
    return CNNCRF_OK;
}

int cnncrf_profile_kernels(char *buf, size_t len)
{
    if (!buf || len == 0) return fail(CNNCRF_EINVAL, "null argument");
    std::lock_guard<std::mutex> lk(g_mu);
    std::string s;
    for (auto &kv : g_recs) s += kv.first + "\n";
    snprintf(buf, len, "%s", s.c_str());
    return CNNCRF_OK;
}

} // extern "C"
