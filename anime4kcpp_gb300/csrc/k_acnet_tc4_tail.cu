// Instantiation of the quad tensor-core kernel's tail part (ACNetLegacy
// layers 5 .. 8 from the activation map, transposed conv, colour merge), in
// a translation unit of its own so it builds in parallel.
#include "k_acnet_tc4.cuh"

namespace acgb {
namespace tcv4 {
template cudaError_t launch_shape<GeoTail, NetLegacyTail<kSplitK>>(int, int, bool, const Params&, int, int, cudaStream_t);
}  // namespace tcv4
}  // namespace acgb
