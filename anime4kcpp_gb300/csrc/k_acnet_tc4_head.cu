// Instantiation of the quad tensor-core kernel's head part (ACNetLegacy
// layers 0 .. 4, writing the 16-bit activation map), in a translation unit
// of its own so it builds in parallel.
#include "k_acnet_tc4.cuh"

namespace acgb {
namespace tcv4 {
template cudaError_t launch_shape<GeoHead, NetLegacyHead<kSplitK>>(int, int, bool, const Params&, int, int, cudaStream_t);
}  // namespace tcv4
}  // namespace acgb
