// Instantiation of the quad tensor-core kernel for tile shape 2 (a
// translation unit of its own to build in parallel).
#include "k_acnet_tc4.cuh"

namespace acgb {
namespace tcv4 {
template cudaError_t launch_shape<GeoQ2, NetLegacy>(int, int, bool, const Params&, int, int, cudaStream_t);
}  // namespace tcv4
}  // namespace acgb
