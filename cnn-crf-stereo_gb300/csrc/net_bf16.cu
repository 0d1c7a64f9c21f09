// net_bf16.cu -- the BF16 tensor-core predict path (placeholder until the
// tcgen05 kernels land).
#include "net.h"

using namespace cnncrf;

int cnncrf_net::predict_bf16(const float *, const float *)
{
    return fail(CNNCRF_EUNSUPPORTED, "BF16 path not built yet");
}
