// Instantiations of the quad tensor-core kernel for its additional tile
// shapes (compiled apart from the default shape to build in parallel).
#include "k_acnet_tc4.cuh"

namespace acgb {
namespace tcv4 {
template cudaError_t launch_shape<GeoQ1, NetLegacy>(int, int, bool, const Params&, int, int, cudaStream_t);
}  // namespace tcv4
}  // namespace acgb
