// Host side of ACNet<8> B4 / B8 in the quad tensor-core kernel
// (k_acnet_tc4.cuh with NetAcn8): B-matrix packing and the launcher.  The
// kernel instantiations live in k_acnet8_tc4_b4.cu and k_acnet8_tc4_b8.cu,
// compiled in parallel with this unit.
#include <cstring>
#include <vector>

#include "k_acnet_tc4.cuh"

namespace acgb {

int* tc_status_buffer();

namespace tcv4 {
cudaError_t launch_acnet8_b4(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream);
cudaError_t launch_acnet8_b8(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream);
cudaError_t launch_acnet8_b8_head(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream);
cudaError_t launch_acnet8_b8_tail(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream);
}  // namespace tcv4

bool acnet8_tc4_supported(int blocks) { return blocks == 4 || blocks == 8; }

void acnet8_tc4_split_tail_shape(int* tw, int* th)
{
    *tw = tcv4::GeoA8B8Tail::TW;
    *th = tcv4::GeoA8B8Tail::TH;
}

void acnet8_tc4_shape(int blocks, int* tw, int* th)
{
    *tw = blocks == 4 ? tcv4::GeoA8B4::TW : tcv4::GeoA8B8::TW;
    *th = blocks == 4 ? tcv4::GeoA8B4::TH : tcv4::GeoA8B8::TH;
}

// Layer 0, the B blocks, then the conv3x3 8 -> 4 tail as an 8-channel layer
// whose outputs 4..7 carry the 16-bit residuals w - hi(w) of outputs 0..3
// (the kernel adds the pairs: FP32-class tail weights).  Reference offsets
// ACNet.hpp:93-114: layer l's kernels at 72 + 576 (l - 1), the tail's 4 x 72
// after them.
void pack_acnet8_tc4_weights(const float* kernels, int blocks, bool bf16, std::vector<uint16_t>& packed)
{
    using namespace tcv4;
    const int nl = blocks + 2;
    packed.assign(static_cast<size_t>(nl) * BL_BYTES / 2, 0);
    pack_quad_layer0(kernels, bf16, packed.data());
    for (int l = 1; l <= blocks; l++)
        pack_quad_conv8(kernels + 72 + 576 * (l - 1), bf16, packed.data() + static_cast<size_t>(l) * BL_BYTES / 2);
    std::vector<float> tail(576, 0.0f);
    const float* kt = kernels + 72 + 576 * blocks;
    for (int i = 0; i < 4 * 72; i++)
    {
        const float hi = bf16 ? __bfloat162float(__float2bfloat16_rn(kt[i])) : __half2float(__float2half_rn(kt[i]));
        tail[i] = hi;
        tail[4 * 72 + i] = kt[i] - hi;
    }
    pack_quad_conv8(tail.data(), bf16, packed.data() + static_cast<size_t>(nl - 1) * BL_BYTES / 2);
}

cudaError_t launch_acnet8_tc4(const float* biases, const float* alphas, int blocks, const void* packed4, bool bf16, int n,
                              const Plane* in, const Plane* out, const Phase2* phase2, int* counter, int ctas,
                              cudaStream_t stream, int per_sm_cap)
{
    using namespace tcv4;
    if (n <= 0) return cudaSuccess;
    if (!acnet8_tc4_supported(blocks) || n > kMaxImages || !packed4 || !counter || ctas <= 0) return cudaErrorInvalidValue;
    int* status = tc_status_buffer();
    if (!status) return cudaErrorMemoryAllocation;
    const int c = in[0].channels, type = in[0].type;
    if (c > 1 && !phase2) return cudaErrorInvalidValue;
    Params p;
    std::memset(&p, 0, sizeof(p));
    p.bw = static_cast<const uint4*>(packed4);
    // biases and PReLU slopes of layer 0 and the blocks at 8 l; the tail's 4 biases after them
    for (int l = 0; l <= blocks; l++)
        for (int k = 0; k < 8; k++)
        {
            p.bias[l][k] = biases[8 * l + k];
            p.alpha[l][k] = alphas[8 * l + k];
        }
    for (int k = 0; k < 4; k++) p.bias[blocks + 1][k] = biases[8 * (blocks + 1) + k];
    if (phase2) p.ph = *phase2;
    int TW = 0, TH = 0;
    acnet8_tc4_shape(blocks, &TW, &TH);
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
    if (blocks == 4) stage_maps<GeoA8B4>(p, n, in);
    else stage_maps<GeoA8B8>(p, n, in);
    err = blocks == 4 ? launch_acnet8_b4(type, c, bf16, p, grid, per_sm_cap, stream)
                      : launch_acnet8_b8(type, c, bf16, p, grid, per_sm_cap, stream);
    if (err == cudaSuccess) count_launch();
    return err;
}

// ACNet<8> B8 in two launches, split at layer 5 (as the ACNetLegacy split):
// the head runs layer 0 and blocks 1-4 and writes block 4's activations
// after PReLU to one 16-bit map per image in `maps` (acnet_tc4_split_map_bytes
// each, in image order); the tail runs blocks 5-8 and the conv 8->4 with the
// nearest add and colour epilogue.  Both windows keep the whole-network B8
// kernel's column parity, so the bytes are the same.  counters: two ints.
cudaError_t launch_acnet8_tc4_split(const float* biases, const float* alphas, int blocks, const void* packed4, bool bf16, int n,
                                    const Plane* in, const Plane* out, const Phase2* phase2, void* maps, int* counters, int ctas,
                                    cudaStream_t stream, int per_sm_cap)
{
    using namespace tcv4;
    constexpr int K = kSplitKA8;
    if (n <= 0) return cudaSuccess;
    if (blocks != 8 || n > kMaxImages || !packed4 || !counters || !maps || ctas <= 0) return cudaErrorInvalidValue;
    int* status = tc_status_buffer();
    if (!status) return cudaErrorMemoryAllocation;
    const int c = in[0].channels, type = in[0].type;
    if (c > 1 && !phase2) return cudaErrorInvalidValue;
    Params H, T;
    std::memset(&H, 0, sizeof(Params));
    std::memset(&T, 0, sizeof(Params));
    H.bw = static_cast<const uint4*>(packed4);
    T.bw = static_cast<const uint4*>(packed4) + static_cast<size_t>(K) * (BL_BYTES / 16);
    // head: layers 0 .. K-1 (bias and PReLU slopes at 8 l)
    for (int l = 0; l < K; l++)
        for (int k = 0; k < 8; k++)
        {
            H.bias[l][k] = biases[8 * l + k];
            H.alpha[l][k] = alphas[8 * l + k];
        }
    // tail: layers K .. blocks with PReLU, then the conv 8->4's four biases
    for (int l = K; l <= blocks; l++)
        for (int k = 0; k < 8; k++)
        {
            T.bias[l - K][k] = biases[8 * l + k];
            T.alpha[l - K][k] = alphas[8 * l + k];
        }
    for (int k = 0; k < 4; k++) T.bias[blocks + 1 - K][k] = biases[8 * (blocks + 1) + k];
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
        H.img[i].tiles_x = (in[i].w + GeoA8B8Head::TW - 1) / GeoA8B8Head::TW;
        H.img[i].tile0 = th;
        th += H.img[i].tiles_x * ((in[i].h + GeoA8B8Head::TH - 1) / GeoA8B8Head::TH);
        T.img[i].in = in[i];
        T.img[i].out = out[i];
        T.img[i].map = m;
        T.img[i].tiles_x = (in[i].w + GeoA8B8Tail::TW - 1) / GeoA8B8Tail::TW;
        T.img[i].tile0 = tt;
        tt += T.img[i].tiles_x * ((in[i].h + GeoA8B8Tail::TH - 1) / GeoA8B8Tail::TH);
    }
    H.nimg = T.nimg = n;
    H.ntiles = th;
    T.ntiles = tt;
    H.tile_counter = counters;
    T.tile_counter = counters + 1;
    H.status = T.status = status;
    stage_maps<GeoA8B8Head>(H, n, in);
    cudaError_t err = cudaMemsetAsync(counters, 0, 2 * sizeof(int), stream);
    if (err != cudaSuccess) return err;
    if ((err = launch_acnet8_b8_head(type, c, bf16, H, th < ctas ? th : ctas, per_sm_cap, stream)) != cudaSuccess) return err;
    count_launch();
    err = launch_acnet8_b8_tail(type, c, bf16, T, tt < ctas ? tt : ctas, per_sm_cap, stream);
    if (err == cudaSuccess) count_launch();
    return err;
}

}  // namespace acgb
