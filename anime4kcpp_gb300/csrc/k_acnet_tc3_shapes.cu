// Instantiations of the persistent tensor-core kernel for the additional
// tile shapes (compiled apart from the default shape to build in parallel).
#include "k_acnet_tc3.cuh"

namespace acgb {
namespace tcv3 {
template cudaError_t launch_shape<Geo1>(int, int, bool, const Params&, int, int, cudaStream_t);
template cudaError_t launch_shape<Geo2>(int, int, bool, const Params&, int, int, cudaStream_t);
}  // namespace tcv3
}  // namespace acgb
