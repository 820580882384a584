// Host side of the quad tensor-core ACNetLegacy kernel (k_acnet_tc4.cuh):
// the B-matrix packing and the launcher.
#include <cstring>
#include <vector>

#include "k_acnet_tc4.cuh"

namespace acgb {

int* tc_status_buffer();

namespace {

uint16_t bits16(float v, bool bf16)
{
    if (bf16)
    {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        return static_cast<uint16_t>((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
    }
    return __half_as_ushort(__float2half_rn(v));
}

}  // namespace

namespace tcv4 {

void pack_quad_conv8(const float* k, bool bf16, uint16_t* out)
{
    static const int off[3][2] = {{0, -1}, {1, 2}, {4, 3}};
    std::memset(out, 0, BL_BYTES);
    for (int dy = 0; dy < 3; dy++)
        for (int j = 0; j < 3; j++)
        {
            uint16_t* ch = out + (3 * dy + j) * (CHUNK_BYTES / 2);
            for (int n = 0; n < 32; n++)
                for (int kk = 0; kk < 16; kk++)
                {
                    const int dx = off[j][kk >> 3] - (n >> 3) + 1;
                    if (dx < 0 || dx > 2) continue;
                    const float w = k[(n & 7) * 72 + (dy * 3 + dx) * 8 + (kk & 7)];
                    ch[((kk >> 3) * 512 + (n >> 3) * 128 + (n & 7) * 16 + (kk & 7) * 2) / 2] = bits16(w, bf16);
                }
        }
}

void pack_quad_layer0(const float* k, bool bf16, uint16_t* out)
{
    auto round16 = [bf16](float v) {
        return bf16 ? __bfloat162float(__float2bfloat16_rn(v)) : __half2float(__float2half_rn(v));
    };
    std::vector<float> k0(576, 0.0f);
    for (int n = 0; n < 8; n++)
        for (int t = 0; t < 9; t++)
        {
            const float v = k[n * 9 + t];
            const float hi = round16(v);
            k0[n * 72 + t * 8 + 0] = hi;
            k0[n * 72 + t * 8 + 1] = hi;
            k0[n * 72 + t * 8 + 2] = v - hi;
        }
    pack_quad_conv8(k0.data(), bf16, out);
}

}  // namespace tcv4

int acnet_tc4_max_images() { return tcv4::kMaxImages; }

void acnet_tc4_shape(int shape, int* tw, int* th)
{
    using namespace tcv4;
    *tw = shape == 1 ? GeoQ1::TW : (shape == 2 ? GeoQ2::TW : Geo0::TW);
    *th = shape == 1 ? GeoQ1::TH : (shape == 2 ? GeoQ2::TH : Geo0::TH);
}

// Layer 0 as an 8-channel layer over the input slots (y_hi, y_lo, y_hi) with
// weights (w_hi, w_hi, w_lo), then the eight 3x3 8->8 layers.
void pack_acnet_tc4_weights(const AcnetLegacyWeights& w, bool bf16, std::vector<uint16_t>& packed)
{
    using namespace tcv4;
    constexpr int NL = NetLegacy::NL;
    packed.assign(static_cast<size_t>(NL) * BL_BYTES / 2, 0);
    pack_quad_layer0(w.k, bf16, packed.data());
    for (int l = 1; l < NL; l++)
        pack_quad_conv8(w.k + 72 + 576 * (l - 1), bf16, packed.data() + static_cast<size_t>(l) * BL_BYTES / 2);
}

// One persistent launch over all tiles of n images (same element type and
// channel count; each output exactly 2x its input).  `counter` is a device
// int the call zeroes on `stream`, `status` the word a timed-out wait sets;
// `ctas` SMs' worth of CTAs drain the queue.
cudaError_t launch_acnet_legacy_tc4_core(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n, const Plane* in,
                                         const Plane* out, const Phase2* phase2, int* counter, int* status, int ctas,
                                         cudaStream_t stream, int per_sm_cap, int shape)
{
    using namespace tcv4;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxImages || !packed4 || !counter || !status || ctas <= 0 || shape < 0 || shape >= kTc4Shapes)
        return cudaErrorInvalidValue;
    const int c = in[0].channels, type = in[0].type;
    if (c > 1 && !phase2) return cudaErrorInvalidValue;
    Params p;
    std::memset(&p, 0, sizeof(p));
    p.bw = static_cast<const uint4*>(packed4);
    for (int i = 0; i < 32; i++) p.k2[i] = wts.k[72 + 576 * 8 + i];
    for (int l = 0; l < NetLegacy::NL; l++)
        for (int k = 0; k < 8; k++) p.bias[l][k] = wts.b[8 * l + k];
    if (phase2) p.ph = *phase2;
    int TW = 0, TH = 0;
    acnet_tc4_shape(shape, &TW, &TH);
    int tiles = 0;
    for (int i = 0; i < n; i++)
    {
        if (in[i].channels != c || in[i].type != type || in[i].w <= 0 || in[i].h <= 0) return cudaErrorInvalidValue;
        p.img[i].in = in[i];
        p.img[i].out = out[i];
        p.img[i].tiles_x = (in[i].w + TW - 1) / TW;
        p.img[i].tile0 = tiles;
        tiles += p.img[i].tiles_x * ((in[i].h + TH - 1) / TH);
    }
    p.nimg = n;
    p.ntiles = tiles;
    p.tile_counter = counter;
    p.status = status;
    cudaError_t err = cudaMemsetAsync(counter, 0, sizeof(int), stream);
    if (err != cudaSuccess) return err;
    const int grid = tiles < ctas ? tiles : ctas;
    switch (shape)
    {
    case 1: stage_maps<GeoQ1>(p, n, in); break;
    case 2: stage_maps<GeoQ2>(p, n, in); break;
    default: stage_maps<Geo0>(p, n, in); break;
    }
    switch (shape)
    {
    case 1: err = launch_shape<GeoQ1, NetLegacy>(type, c, bf16, p, grid, per_sm_cap, stream); break;
    case 2: err = launch_shape<GeoQ2, NetLegacy>(type, c, bf16, p, grid, per_sm_cap, stream); break;
    default: err = launch_shape<Geo0, NetLegacy>(type, c, bf16, p, grid, per_sm_cap, stream); break;
    }
    if (err == cudaSuccess) count_launch();
    return err;
}

void acnet_tc4_split_tail_shape(int* tw, int* th)
{
    *tw = tcv4::GeoTail::TW;
    *th = tcv4::GeoTail::TH;
}

size_t acnet_tc4_split_map_bytes(int w, int h)
{
    return static_cast<size_t>((w * 16 + 255) & ~255) * h;
}

// The network in two launches (fusion depth 5 + 4): the head runs layers
// 0 .. 4 over 54x54 tiles and writes layer 4's 16-bit activations (16 bytes
// per pixel) to one map per image in `maps` (acnet_tc4_split_map_bytes each,
// 256-byte aligned, in image order); the tail reads them over 46x57 tiles
// and runs layers 5 .. 8, the transposed conv and the colour merge.  The
// tail reads exactly the values the whole-network kernel keeps in shared
// memory, and both parts' windows put every image column at the whole-
// network windows' column parity (the grouping of the taps in the MMAs), so
// the bytes are the same.  counters[0] / [1]: the two launches' tile
// counters (zeroed here on `stream`).
cudaError_t launch_acnet_legacy_tc4_split(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n,
                                          const Plane* in, const Plane* out, const Phase2* phase2, void* maps,
                                          int* counters, int ctas, cudaStream_t stream, int per_sm_cap)
{
    using namespace tcv4;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxImages || !packed4 || !counters || !maps || ctas <= 0) return cudaErrorInvalidValue;
    int* status = tc_status_buffer();
    if (!status) return cudaErrorMemoryAllocation;
    const int c = in[0].channels, type = in[0].type;
    if (c > 1 && !phase2) return cudaErrorInvalidValue;
    Params H, T;
    std::memset(&H, 0, sizeof(Params));
    std::memset(&T, 0, sizeof(Params));
    H.bw = static_cast<const uint4*>(packed4);
    T.bw = static_cast<const uint4*>(packed4) + static_cast<size_t>(kSplitK) * (BL_BYTES / 16);
    for (int l = 0; l < kSplitK; l++)
        for (int k = 0; k < 8; k++) H.bias[l][k] = wts.b[8 * l + k];
    for (int l = 0; l < 9 - kSplitK; l++)
        for (int k = 0; k < 8; k++) T.bias[l][k] = wts.b[8 * (kSplitK + l) + k];
    for (int i = 0; i < 32; i++) T.k2[i] = wts.k[72 + 576 * 8 + i];
    if (phase2) T.ph = *phase2;
    size_t off = 0;
    int th = 0, tt = 0;
    for (int i = 0; i < n; i++)
    {
        if (in[i].channels != c || in[i].type != type || in[i].w <= 0 || in[i].h <= 0) return cudaErrorInvalidValue;
        Plane m;
        m.ptr = static_cast<char*>(maps) + off;
        m.w = in[i].w;
        m.h = in[i].h;
        m.pitch = (in[i].w * 16 + 255) & ~255;
        m.channels = 8;
        m.type = type;
        off += acnet_tc4_split_map_bytes(in[i].w, in[i].h);
        H.img[i].in = in[i];
        H.img[i].out = m;
        H.img[i].map = m;
        H.img[i].tiles_x = (in[i].w + GeoHead::TW - 1) / GeoHead::TW;
        H.img[i].tile0 = th;
        th += H.img[i].tiles_x * ((in[i].h + GeoHead::TH - 1) / GeoHead::TH);
        T.img[i].in = in[i];
        T.img[i].out = out[i];
        T.img[i].map = m;
        T.img[i].tiles_x = (in[i].w + GeoTail::TW - 1) / GeoTail::TW;
        T.img[i].tile0 = tt;
        tt += T.img[i].tiles_x * ((in[i].h + GeoTail::TH - 1) / GeoTail::TH);
    }
    H.nimg = T.nimg = n;
    H.ntiles = th;
    T.ntiles = tt;
    H.tile_counter = counters;
    T.tile_counter = counters + 1;
    H.status = T.status = status;
    stage_maps<GeoHead>(H, n, in);
    cudaError_t err = cudaMemsetAsync(counters, 0, 2 * sizeof(int), stream);
    if (err != cudaSuccess) return err;
    err = launch_shape<GeoHead, NetLegacyHead<kSplitK>>(type, c, bf16, H, th < ctas ? th : ctas, per_sm_cap, stream);
    if (err != cudaSuccess) return err;
    count_launch();
    err = launch_shape<GeoTail, NetLegacyTail<kSplitK>>(type, c, bf16, T, tt < ctas ? tt : ctas, per_sm_cap, stream);
    if (err == cudaSuccess) count_launch();
    return err;
}

cudaError_t launch_acnet_legacy_tc4(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n, const Plane* in,
                                    const Plane* out, const Phase2* phase2, int* counter, int ctas, cudaStream_t stream,
                                    int per_sm_cap, int shape)
{
    int* status = tc_status_buffer();
    if (!status) return cudaErrorMemoryAllocation;
    return launch_acnet_legacy_tc4_core(wts, packed4, bf16, n, in, out, phase2, counter, status, ctas, stream, per_sm_cap,
                                        shape);
}

}  // namespace acgb
