// ACNet<8> B8 split network, head part (layer 0 and blocks 1-4) of the quad
// tensor-core kernel, in a translation unit of its own so it compiles in
// parallel.
#include "k_acnet_tc4.cuh"

namespace acgb {
namespace tcv4 {

cudaError_t launch_acnet8_b8_head(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    return launch_shape<GeoA8B8Head, NetAcn8Head<8, kSplitKA8>>(type, c, bf16, p, grid, per_sm_cap, stream);
}

}  // namespace tcv4
}  // namespace acgb
