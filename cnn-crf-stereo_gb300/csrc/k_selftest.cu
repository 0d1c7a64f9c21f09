// k_selftest.cu -- a self-test of the bounded device waits and of the error
// path they feed (no reference counterpart: the reference's kernels have no
// device-side waits, and its errors end the process).
//
// Every mbarrier wait in the tensor-core kernels is bounded (tc::mbar_wait): it
// gives up after a number of polls, and the kernel then raises a device error
// flag that the host turns into CNNCRF_ETIMEOUT instead of hanging.  This probe
// runs that same wait on a barrier of its own -- one that nothing arrives on
// unless `arrive` is set -- with a caller-chosen poll limit, sets the flag when
// the wait gives up, and reports the status through the same mapping.  It moves
// no data: no asynchronous copies, no tensor memory, nothing to drain, so a wait
// that runs out leaves the context usable.
#include "common.h"
#include "kernels.h"
#include "tc_util.cuh"

namespace cnncrf {
namespace k {

namespace {

__global__ void k_wait_probe(int *err, uint32_t polls, int arrive)
{
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        abort_flag = 0;
        tc::mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (arrive) tc::mbar_arrive(&bar);
        if (!tc::mbar_wait(&bar, 0, &abort_flag, polls)) atomicExch(err, 1);
    }
}

} // namespace

int selftest_bounded_wait(int polls, int arrive, cudaStream_t st)
{
    if (polls < 1 || polls > (1 << 20)) return fail(CNNCRF_EINVAL, "selftest: polls %d outside 1..2^20", polls);
    DevBuf flag;
    CNNCRF_TRY(flag.reserve(sizeof(int)));
    CNNCRF_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), st));
    {
        CNNCRF_PROF("wait_probe", st);
        k_wait_probe<<<1, 32, 0, st>>>(flag.as<int>(), (uint32_t)polls, arrive ? 1 : 0);
    }
    CNNCRF_CHECK_LAUNCH();
    int h = 0;
    CNNCRF_CUDA(cudaMemcpyAsync(&h, flag.get(), sizeof(int), cudaMemcpyDeviceToHost, st));
    CNNCRF_CUDA(cudaStreamSynchronize(st));
    if (h) return fail(CNNCRF_ETIMEOUT, "selftest: a bounded wait gave up after %d polls", polls);
    return CNNCRF_OK;
}

} // namespace k
} // namespace cnncrf
