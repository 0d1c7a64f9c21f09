// k_crf_r4.cu -- the CRF chain pass with a 4-step prefetch ring (the
// kernels of k_crf_chain.cuh instantiated for RING = 4; k_crf.cu holds the
// 8-step ones and the solver around them).  A shallower ring leaves more
// shared memory for resident chains; which depth is faster depends on the
// label count and the chain length, and the tile tuner measures it.
// Compiled with --fmad=false like k_crf.cu: the labels equal the oracle's.
#include "k_crf_chain.cuh"

namespace cnncrf {
namespace k {

int crf_pass_ring4(const CrfPassArgs &a, bool hpass, int delta, int wpb, cudaStream_t st)
{
    return launch_pass_any<4>(a, hpass, delta, wpb, st);
}

} // namespace k
} // namespace cnncrf
