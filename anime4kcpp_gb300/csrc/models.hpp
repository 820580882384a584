// Model selection and parameters for the GB300 backend.
//
// Families: ACNetLegacy (trained parameters of the reference, variants GAN
// and HDN0..3), ACNet<8> (trained parameters of the reference, B4/8/18 x
// {normal, HDN, Box, Box-HDN}), ArtCNN<16/32> (C4 x {normal, DN, DS}),
// FSRCNNX<8/16> (B4 x {normal, DistortPlus}), all with the reference's trained
// parameters, and ARNet<8> (B8/16/32/64 x {normal, HDN, Box, Box-HDN};
// seeded synthetic parameters because the reference's trained ARNet
// parameters are not distributed with its source).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace acgb {

enum class Family { ACNetLegacy, ARNet, ACNet8, ArtCNN, FSRCNNX };

struct ModelSpec
{
    Family family = Family::ACNetLegacy;
    int variant = 0;  // ACNetLegacy: 0 GAN, 1..4 HDN0..3
    int blocks = 0;   // ARNet: 8, 16, 32, 64; ACNet<8>: 4, 8, 18
    int kind = 0;     // ARNet, ACNet<8>: 0 normal, 1 HDN, 2 Box, 3 Box-HDN; ArtCNN: 0 normal, 1 DN, 2 DS;
                      // FSRCNNX: 0 normal, 1 DistortPlus
    int channels = 8; // feature channels F (ArtCNN 16/32, FSRCNNX 8/16, else 8)
    std::string name;
};

// Parses a model string like core/src/processor/Processor.cpp:26-187 does
// for every family of the reference (ACNetLegacy, ACNet<8>, ARNet<8>,
// ArtCNN<16/32>, FSRCNNX<8/16>).  Like the reference it accepts every
// string (anything unrecognised is ACNetLegacy GAN), so it returns true and
// leaves `error` alone; the flag and message stay for the callers' uniform
// failure path.
bool parse_model(const char* model, ModelSpec& spec, std::string& error);

struct ModelParams
{
    std::vector<float> kernels, biases, alphas;
};

// Parameters in the reference's NHWC blob layout (ACNet.hpp:34-60 and
// :63-116, ARNet.hpp:26-70).
const ModelParams& model_params(const ModelSpec& spec);

// Seed of the synthetic ARNet parameters of a variant.
constexpr uint64_t kArnetSeedBase = 0x41524E6574000000ull;
void arnet_synthetic_params(int blocks, uint64_t seed, ModelParams& out);

}  // namespace acgb
