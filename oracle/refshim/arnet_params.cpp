// Definitions of the ARNet parameter arrays declared by the ARNet.p stub,
// filled before main() with the seeded synthetic generator of
// oracle/acoracle.c (orc_arnet_synth).  Seed of a variant:
//   0x41524E6574000000 + 16 * blocks + kind   (kind: 0 normal, 1 HDN, 2 Box, 3 Box-HDN)
// Shapes follow core/include/AC/Core/Model/ARNet.hpp:26-33 for F = 8.
#include <cstdint>

extern "C" int orc_arnet_synth(int blocks, std::uint64_t seed, float* kernels, float* biases, float* alphas);

namespace ac::core::model::param
{
#define AR_DEFINE(B, SUF) \
    float ARNet_F8B##B##SUF##_NHWC_kernels[72 + 576 * 2 * B + 64 + 288]; \
    float ARNet_F8B##B##SUF##_NHWC_biases[8 + 8 * (2 * B + 1) + 4]; \
    float ARNet_F8B##B##SUF##_NHWC_alphas[8 * (B + 1)];
#define AR_ALL(B) AR_DEFINE(B, ) AR_DEFINE(B, _HDN) AR_DEFINE(B, _Box) AR_DEFINE(B, _Box_HDN)
    AR_ALL(8) AR_ALL(16) AR_ALL(32) AR_ALL(64)
}

namespace
{
    struct Filler
    {
        Filler()
        {
            using namespace ac::core::model::param;
            constexpr std::uint64_t base = 0x41524E6574000000ull;
#define AR_FILL(B, SUF, KIND) orc_arnet_synth(B, base + 16 * B + KIND, ARNet_F8B##B##SUF##_NHWC_kernels, ARNet_F8B##B##SUF##_NHWC_biases, ARNet_F8B##B##SUF##_NHWC_alphas);
#define AR_FILL_ALL(B) AR_FILL(B, , 0) AR_FILL(B, _HDN, 1) AR_FILL(B, _Box, 2) AR_FILL(B, _Box_HDN, 3)
            AR_FILL_ALL(8) AR_FILL_ALL(16) AR_FILL_ALL(32) AR_FILL_ALL(64)
        }
    } filler;
}
