// Model string parsing and parameter tables.
#include "models.hpp"

#include <algorithm>
#include <cctype>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

namespace acgb {

// Generated at build time from weights/acnet_legacy.bin (see build.py):
// 5 variants (GAN, HDN0..3) x (4712 kernel + 72 bias) float32 bit patterns.
extern const uint32_t kAcnetLegacyBlob[];
extern const int kAcnetLegacyVariants;
extern const int kAcnetLegacyKernels;
extern const int kAcnetLegacyBiases;
// Generated at build time from weights/acnet8.bin: word 0 the variant count
// (12), then per variant a header {blocks, kernel floats, bias floats, alpha
// floats} and the floats.
extern const uint32_t kAcnet8Blob[];
extern const int kAcnet8Words;
// Generated at build time from weights/artcnn_fsrcnnx.bin: word 0 the variant
// count (10), then per variant a header {family (1 ArtCNN, 2 FSRCNNX), F,
// blocks, kind, kernel floats, bias floats, alpha floats} and the floats.
extern const uint32_t kArtFsrBlob[];
extern const int kArtFsrWords;

bool parse_model(const char* model, ModelSpec& spec, std::string& /*error*/)
{
    std::string s = model ? model : "";
    for (char& ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    spec = ModelSpec{};
    spec.name = model ? model : "";
    auto has = [&](const char* t) { return s.find(t) != std::string::npos; };
    if (has("fsrcnnx"))
    {
        // Processor.cpp:40-55: f16 picks FSRCNNX<16>; "distort" or "dp" the DistortPlus variant
        spec.family = Family::FSRCNNX;
        spec.channels = has("f16") ? 16 : 8;
        spec.blocks = 4;
        spec.kind = (has("distort") || has("dp")) ? 1 : 0;
        return true;
    }
    if (has("artcnn"))
    {
        // Processor.cpp:56-74: f32 picks ArtCNN<32>; "dn" then "ds" pick the variant
        spec.family = Family::ArtCNN;
        spec.channels = has("f32") ? 32 : 16;
        spec.blocks = 4;
        spec.kind = has("dn") ? 1 : (has("ds") ? 2 : 0);
        return true;
    }
    if (has("arnet"))
    {
        spec.family = Family::ARNet;
        spec.blocks = 8;
        // Processor.cpp:82-124 checks b8 before b16/b32/b64.
        if (has("b8")) spec.blocks = 8;
        else if (has("b16")) spec.blocks = 16;
        else if (has("b32")) spec.blocks = 32;
        else if (has("b64")) spec.blocks = 64;
        spec.kind = (has("box") ? 2 : 0) + (has("hdn") ? 1 : 0);
        return true;
    }
    if (has("acnet"))
    {
        if (has("legacy"))
        {
            spec.family = Family::ACNetLegacy;
            spec.variant = 0;
            if (has("hdn"))
            {
                // Processor.cpp:130-141: first digit 0..3 found picks HDN0..3.
                spec.variant = 1;
                for (char ch : s)
                    if (ch >= '0' && ch <= '3')
                    {
                        spec.variant = 1 + (ch - '0');
                        break;
                    }
            }
            return true;
        }
        // ACNet<8> (Processor.cpp:146-184): every branch checks b4, then
        // b8, then b18, with B8 the default; box and hdn pick the kind.
        spec.family = Family::ACNet8;
        spec.blocks = 8;
        if (has("b4")) spec.blocks = 4;
        else if (has("b8")) spec.blocks = 8;
        else if (has("b18")) spec.blocks = 18;
        spec.kind = (has("box") ? 2 : 0) + (has("hdn") ? 1 : 0);
        return true;
    }
    // Processor.cpp:186: anything else is ACNetLegacy GAN.
    spec.family = Family::ACNetLegacy;
    spec.variant = 0;
    return true;
}

namespace {

uint64_t splitmix64(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// 24-bit uniform in [-1, 1): exact in float.
float uniform_pm1(uint64_t& s)
{
    uint64_t r = splitmix64(s) >> 40;
    return static_cast<float>(r) * (1.0f / 8388608.0f) - 1.0f;
}

}  // namespace

void arnet_synthetic_params(int blocks, uint64_t seed, ModelParams& out)
{
    const int nconv = 2 * blocks;
    const int kl = 72 + 576 * nconv + 64 + 288;
    const int bl = 8 + 8 * (nconv + 1) + 4;
    const int al = 8 * (blocks + 1);
    out.kernels.resize(kl);
    out.biases.resize(bl);
    out.alphas.resize(al);
    uint64_t s = seed;
    for (int i = 0; i < kl; i++)
    {
        float scale;
        if (i < 72) scale = 0.5f;                            // head 1 -> 8
        else if (i < 72 + 576 * nconv) scale = 0.12f;         // body 3x3 8 -> 8
        else if (i < 72 + 576 * nconv + 64) scale = 0.2f;    // tail 1x1 8 -> 8
        else scale = 0.02f;                                   // upscale 3x3 8 -> 4
        out.kernels[i] = uniform_pm1(s) * scale;
    }
    for (int i = 0; i < bl; i++) out.biases[i] = uniform_pm1(s) * 0.01f;
    for (int i = 0; i < al; i++) out.alphas[i] = (uniform_pm1(s) + 1.0f) * 0.125f;
}

const ModelParams& model_params(const ModelSpec& spec)
{
    static std::mutex m;
    static std::map<std::tuple<int, int, int, int>, ModelParams> cache;
    std::lock_guard<std::mutex> lock(m);
    const auto key = spec.family == Family::ACNetLegacy
                         ? std::make_tuple(static_cast<int>(spec.family), spec.variant, 0, 0)
                         : std::make_tuple(static_cast<int>(spec.family), spec.blocks, spec.kind, spec.channels);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    ModelParams p;
    if (spec.family == Family::ACNetLegacy)
    {
        const int per = kAcnetLegacyKernels + kAcnetLegacyBiases;
        const uint32_t* base = kAcnetLegacyBlob + static_cast<size_t>(spec.variant) * per;
        p.kernels.resize(kAcnetLegacyKernels);
        p.biases.resize(kAcnetLegacyBiases);
        std::memcpy(p.kernels.data(), base, sizeof(float) * kAcnetLegacyKernels);
        std::memcpy(p.biases.data(), base + kAcnetLegacyKernels, sizeof(float) * kAcnetLegacyBiases);
    }
    else if (spec.family == Family::ACNet8)
    {
        // variants in blob order: blocks 4, 8, 18, each as normal, HDN, Box, Box-HDN
        const int want = (spec.blocks == 4 ? 0 : spec.blocks == 8 ? 1 : 2) * 4 + spec.kind;
        size_t at = 1;
        for (int v = 0; v <= want && v < static_cast<int>(kAcnet8Blob[0]); v++)
        {
            const uint32_t* h = kAcnet8Blob + at;
            const size_t nk = h[1], nb = h[2], na = h[3];
            if (v == want)
            {
                p.kernels.resize(nk);
                p.biases.resize(nb);
                p.alphas.resize(na);
                std::memcpy(p.kernels.data(), h + 4, sizeof(float) * nk);
                std::memcpy(p.biases.data(), h + 4 + nk, sizeof(float) * nb);
                std::memcpy(p.alphas.data(), h + 4 + nk + nb, sizeof(float) * na);
            }
            at += 4 + nk + nb + na;
        }
    }
    else if (spec.family == Family::ArtCNN || spec.family == Family::FSRCNNX)
    {
        const uint32_t fam = spec.family == Family::ArtCNN ? 1u : 2u;
        size_t at = 1;
        for (uint32_t v = 0; v < kArtFsrBlob[0]; v++)
        {
            const uint32_t* h = kArtFsrBlob + at;
            const size_t nk = h[4], nb = h[5], na = h[6];
            if (h[0] == fam && static_cast<int>(h[1]) == spec.channels && static_cast<int>(h[3]) == spec.kind)
            {
                p.kernels.resize(nk);
                p.biases.resize(nb);
                p.alphas.resize(na);
                std::memcpy(p.kernels.data(), h + 7, sizeof(float) * nk);
                std::memcpy(p.biases.data(), h + 7 + nk, sizeof(float) * nb);
                if (na) std::memcpy(p.alphas.data(), h + 7 + nk + nb, sizeof(float) * na);
                break;
            }
            at += 7 + nk + nb + na;
        }
    }
    else
    {
        arnet_synthetic_params(spec.blocks, kArnetSeedBase + 16ull * spec.blocks + spec.kind, p);
    }
    return cache.emplace(key, std::move(p)).first->second;
}

}  // namespace acgb
