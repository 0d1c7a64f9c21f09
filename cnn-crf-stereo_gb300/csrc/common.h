// common.h -- error plumbing, device buffers and kernel-launch helpers shared
// by the host code of libcnncrf (plain C++; included by .cu and .cpp files).
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cnncrf.h"

namespace cnncrf {

// Record a failure for cnncrf_last_error() and return its status code.
int fail(int status, const char *fmt, ...);
void clear_error();

#define CNNCRF_CUDA(call)                                                                      \
    do {                                                                                       \
        cudaError_t e__ = (call);                                                              \
        if (e__ != cudaSuccess)                                                                \
            return ::cnncrf::fail(CNNCRF_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,      \
                                  cudaGetErrorString(e__));                                    \
    } while (0)

#define CNNCRF_CHECK_LAUNCH() CNNCRF_CUDA(cudaGetLastError())

#define CNNCRF_TRY(expr)                                                                       \
    do {                                                                                       \
        int s__ = (expr);                                                                      \
        if (s__ != CNNCRF_OK) return s__;                                                      \
    } while (0)

// Owning device allocation (cudaMalloc / cudaFree), 256-byte aligned.
class DevBuf {
  public:
    DevBuf() = default;
    ~DevBuf() { release(); }
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr, o.n_ = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) {
            release();
            p_ = o.p_, n_ = o.n_;
            o.p_ = nullptr, o.n_ = 0;
        }
        return *this;
    }
    // (Re)allocate to at least `bytes`; keeps the buffer when large enough.
    int reserve(size_t bytes)
    {
        if (bytes <= n_ && p_) return CNNCRF_OK;
        release();
        if (bytes == 0) return CNNCRF_OK;
        cudaError_t e = cudaMalloc(&p_, bytes);
        if (e != cudaSuccess) {
            p_ = nullptr;
            (void)cudaGetLastError();
            return fail(CNNCRF_ENOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
        }
        n_ = bytes;
        return CNNCRF_OK;
    }
    void release()
    {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    template <class T> T *as() const { return static_cast<T *>(p_); }
    void *get() const { return p_; }
    size_t size() const { return n_; }

  private:
    void *p_ = nullptr;
    size_t n_ = 0;
};

inline int ceil_div(long a, long b) { return (int)((a + b - 1) / b); }

// Kernel-launch instrumentation.  Every launch site is wrapped in a
// CNNCRF_PROF scope: it counts the launch, opens an NVTX range named after
// the kernel in the "cnncrf" domain (a no-op unless a tool such as ncu with
// --nvtx is attached) and, while timing is enabled (cnncrf_profile_enable),
// records a CUDA event pair around it on the launching stream, filed under
// the kernel's name.
class Prof {
  public:
    Prof(const char *name, cudaStream_t st);
    ~Prof();

  private:
    const char *name_;
    cudaStream_t st_;
    cudaEvent_t a_ = nullptr;
};
#define CNNCRF_PROF(name, st) ::cnncrf::Prof prof__(name, st)

// An NVTX range around a whole stage of an API call (the volume, the CRF,
// the refinement, a batch run, a training step), nesting the kernels' ranges.
class Range {
  public:
    explicit Range(const char *name);
    ~Range();
};
#define CNNCRF_RANGE(name) ::cnncrf::Range range__(name)

} // namespace cnncrf
