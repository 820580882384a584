// Host side of the persistent tensor-core ACNetLegacy kernel
// (k_acnet_tc3.cuh): the default tile shape's instantiation, the launchers
// and the allocation-free entry's static scratch.
#include <cstring>
#include <mutex>

#include "k_acnet_tc3.cuh"

namespace acgb {

int* tc_status_buffer();

int acnet_tc3_max_images() { return tcv3::kMaxImages; }

// B matrices of the persistent kernel: layer 0 as an 8-channel layer over
// the input slots (y_hi, y_lo, y_hi) with weights (w_hi, w_hi, w_lo), then
// the eight 3x3 8->8 layers, each in the pair layout of pack_pair_conv8.
void pack_acnet_tc3_weights(const AcnetLegacyWeights& w, bool bf16, std::vector<uint16_t>& packed)
{
    using namespace tcv3;
    packed.assign(static_cast<size_t>(B_BYTES) / 2, 0);
    auto round16 = [bf16](float v) {
        return bf16 ? __bfloat162float(__float2bfloat16_rn(v)) : __half2float(__float2half_rn(v));
    };
    std::vector<float> k0(576, 0.0f);
    for (int n = 0; n < 8; n++)
        for (int t = 0; t < 9; t++)
        {
            const float v = w.k[n * 9 + t];  // layer 0: k[n * 9 + tap] (ACNet.hpp:48-60)
            const float hi = round16(v);
            k0[n * 72 + t * 8 + 0] = hi;
            k0[n * 72 + t * 8 + 1] = hi;
            k0[n * 72 + t * 8 + 2] = v - hi;
        }
    pack_pair_conv8(k0.data(), bf16, packed.data());
    for (int l = 1; l < NL; l++)
        pack_pair_conv8(w.k + 72 + 576 * (l - 1), bf16, packed.data() + static_cast<size_t>(l) * BL_BYTES / 2);
}

void acnet_tc3_shape(int shape, int* tw, int* th)
{
    using namespace tcv3;
    switch (shape)
    {
    case 1: *tw = Geo1::TW, *th = Geo1::TH; break;
    case 2: *tw = Geo2::TW, *th = Geo2::TH; break;
    default: *tw = Geo0::TW, *th = Geo0::TH; break;
    }
}

namespace {

// One persistent launch over all tiles of n images; `counter` (zeroed here
// on `stream`) is the tile queue, `status` the word a timed-out wait sets.
cudaError_t launch_tc3(const AcnetLegacyWeights& wts, const void* packed2, bool bf16, int n, const Plane* in, const Plane* out,
                       const Phase2* phase2, int* counter, int* status, int ctas, cudaStream_t stream, int shape,
                       int per_sm_cap)
{
    using namespace tcv3;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxImages || !packed2 || !counter || !status || ctas <= 0 || shape < 0 || shape >= kTc3Shapes)
        return cudaErrorInvalidValue;
    int TW = 0, TH = 0;
    acnet_tc3_shape(shape, &TW, &TH);
    const int c = in[0].channels, type = in[0].type;
    if (c > 1 && !phase2) return cudaErrorInvalidValue;
    Params p;
    std::memset(&p, 0, sizeof(p));
    p.bw = static_cast<const uint4*>(packed2);
    for (int i = 0; i < 32; i++) p.k2[i] = wts.k[72 + 576 * 8 + i];
    for (int l = 0; l < NL; l++)
        for (int k = 0; k < 8; k++) p.bias[l][k] = wts.b[8 * l + k];
    if (phase2) p.ph = *phase2;
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
    case 1: err = launch_shape<Geo1>(type, c, bf16, p, grid, per_sm_cap, stream); break;
    case 2: err = launch_shape<Geo2>(type, c, bf16, p, grid, per_sm_cap, stream); break;
    default: err = launch_shape<Geo0>(type, c, bf16, p, grid, per_sm_cap, stream); break;
    }
    if (err == cudaSuccess) count_launch();
    return err;
}

// Scratch of the allocation-free entry: word 0 is the tile-queue counter,
// word 1 the status word; a call zeroes both on its stream before the launch
// and uses 8 of the 256 bytes whatever the batch.  Calls that overlap in
// time on one device share it and race.
constexpr int kNoAllocScratchInts = 64;
constexpr int kNoAllocMaxDevices = 64;
static __device__ __align__(256) int g_tc3_noalloc_scratch[kNoAllocScratchInts];

// Device address of the scratch on the current device, resolved once per
// device (the set-up step of the first call on that device).
cudaError_t noalloc_scratch(int** out)
{
    static std::mutex m;
    static int* addr[kNoAllocMaxDevices] = {};
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(m);
    if (!addr[dev])
    {
        void* p = nullptr;
        err = cudaGetSymbolAddress(&p, g_tc3_noalloc_scratch);
        if (err != cudaSuccess) return err;
        addr[dev] = static_cast<int*>(p);
    }
    *out = addr[dev];
    return cudaSuccess;
}

}  // namespace

// One persistent launch over all tiles of n images (same element type and
// channel count; each output exactly 2x its input).  `counter` is a device
// int the call zeroes on `stream` before the launch; `ctas` SMs' worth of
// CTAs (one or two per SM, as many as fit) drain the queue.
cudaError_t launch_acnet_legacy_tc3(const AcnetLegacyWeights& wts, const void* packed2, bool bf16, int n, const Plane* in,
                                    const Plane* out, const Phase2* phase2, int* counter, int ctas, cudaStream_t stream,
                                    int shape, int per_sm_cap)
{
    int* status = tc_status_buffer();
    if (!status) return cudaErrorMemoryAllocation;
    return launch_tc3(wts, packed2, bf16, n, in, out, phase2, counter, status, ctas, stream, shape, per_sm_cap);
}

// The same launch with its counter and status word in the file's static
// scratch: allocates no memory (first call per device: symbol look-up).
cudaError_t launch_acnet_legacy_tc3_noalloc(const AcnetLegacyWeights& wts, const void* packed2, bool bf16, int n,
                                            const Plane* in, const Plane* out, const Phase2* phase2, int ctas,
                                            cudaStream_t stream)
{
    int* s = nullptr;
    cudaError_t err = noalloc_scratch(&s);
    if (err != cudaSuccess) return err;
    if ((err = cudaMemsetAsync(s, 0, 2 * sizeof(int), stream)) != cudaSuccess) return err;
    return launch_tc3(wts, packed2, bf16, n, in, out, phase2, s, s + 1, ctas, stream, 0, 2);
}

// The quad kernel's launch over the same scratch (counter and status word).
cudaError_t launch_acnet_legacy_tc4_noalloc(const AcnetLegacyWeights& wts, const void* packed4, bool bf16, int n,
                                            const Plane* in, const Plane* out, const Phase2* phase2, int ctas,
                                            cudaStream_t stream)
{
    int* s = nullptr;
    cudaError_t err = noalloc_scratch(&s);
    if (err != cudaSuccess) return err;
    if ((err = cudaMemsetAsync(s, 0, 2 * sizeof(int), stream)) != cudaSuccess) return err;
    return launch_acnet_legacy_tc4_core(wts, packed4, bf16, n, in, out, phase2, s, s + 1, ctas, stream, 2);
}

// Status word of the allocation-free launches on the current device: 0, or
// 1 when a bounded wait gave up.  Read it after the stream synchronised.
cudaError_t acnet_tc3_noalloc_status(int* value)
{
    int* s = nullptr;
    cudaError_t err = noalloc_scratch(&s);
    if (err != cudaSuccess) return err;
    return cudaMemcpy(value, s + 1, sizeof(int), cudaMemcpyDeviceToHost);
}

}  // namespace acgb
