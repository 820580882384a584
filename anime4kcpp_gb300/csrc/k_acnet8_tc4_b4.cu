// ACNet<8> B4 instantiations of the quad tensor-core kernel (k_acnet_tc4.cuh),
// in a translation unit of their own so they compile in parallel.
#include "k_acnet_tc4.cuh"

namespace acgb {
namespace tcv4 {

cudaError_t launch_acnet8_b4(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    return launch_shape<GeoA8B4, NetAcn8<4>>(type, c, bf16, p, grid, per_sm_cap, stream);
}

}  // namespace tcv4
}  // namespace acgb
