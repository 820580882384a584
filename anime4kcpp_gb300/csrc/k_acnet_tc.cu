// Tensor-core form of the layer-fused ACNetLegacy pass (placeholder until the
// tcgen05 kernel lands).
#include "kernels.hpp"

namespace acgb {

void pack_acnet_tc_weights(const AcnetLegacyWeights&, bool, std::vector<uint16_t>& packed) { packed.assign(8, 0); }

cudaError_t launch_acnet_legacy_tc(const AcnetLegacyWeights&, const void*, bool, const Plane&, const Plane&, cudaStream_t)
{
    return cudaErrorNotSupported;
}

}  // namespace acgb
