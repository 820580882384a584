// ARNet<8> x2 pass in a tensor-core form (FP16 or BF16 operands, FP32
// accumulation), one launch per layer.
//
// Network and CPU order as k_arnet_fp32.cu (core/include/AC/Core/Model/ARNet.hpp:16-72,
// core/src/processor/cpu/CPUProcessor.cpp:1464-1491, layer templates
// core/internal/AC/Core/Internal/Processor/CPU/Common.hpp:116-197,223-342).
// The first layer (conv 1->8) and the last (conv 8->4 + pixel shuffle +
// nearest input) stay FP32 on CUDA cores; the 2B 3x3 8->8 convolutions run on
// tcgen05 as the pair-interleaved implicit GEMM of the ACNetLegacy kernels:
// one GEMM row = two adjacent pixels (N = 16), K = 3 tap rows x 4 pixels x 8
// channels read as shifted views of an even/odd plane pair in shared memory,
// six 128x16x16 MMAs per 128 pairs, accumulators in tensor memory.
//
// Between layers the 8-channel maps live in HBM as [h][w][8] 16-bit values
// (16 bytes per pixel, as the reference's CUDA processor keeps FP16
// intermediates, Kernel.cu:284-333).  A CTA of 128 threads computes a 62x30
// tile from a 64x32 window (halo 1, clamped to the map's edge): 2,048 pixels
// = 1,024 pairs = 8 blocks of 128 GEMM rows in 128 tensor-memory columns, four
// CTAs per SM.  The epilogue adds the bias in FP32 and applies the layer's
// ending: PReLU; 0.2 x conv + the block input (residual); or, for the last
// block, the residual followed by the 1x1 conv 8->8 + PReLU + the head's
// features.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"

namespace acgb {
namespace arnettc {

constexpr int TW = 62, TH = 30;
constexpr int WW = TW + 2, WH = TH + 2;  // 64 x 32 window
constexpr int PPR = WW / 2;
constexpr int NBLK = WW * WH / 2 / 128;  // 8
constexpr int PADP = 40;
constexpr int PLANE_BYTES = (PADP + NBLK * 128 + PADP) * 16;
constexpr int B_BYTES = 12 * 256;  // one layer's packed weights
constexpr int THREADS = 128;
constexpr uint32_t TMEM_COLS = 128;
constexpr int SMEM = 2 * PLANE_BYTES + B_BYTES + 64;
// Shared memory requested per CTA: at least a fifth of the SM's, so that at
// most four CTAs (4 x 128 tensor-memory columns) are resident on an SM.
constexpr int SMEM_REQ = SMEM > 48 * 1024 ? SMEM : 48 * 1024;
constexpr uint64_t kWaitNs = 2000000000ull;
static_assert(WW * WH / 2 == NBLK * 128, "the window is whole pair blocks");
static_assert(PADP >= PPR + 2, "taps of the first and last rows stay inside the planes");

enum Mode
{
    kPReLU = 0,     // prelu(conv + b)
    kResidual = 1,  // 0.2 * (conv + b) + skip
    kTail = 2,      // prelu(1x1(0.2 * (conv + b) + skip) + b1) + feat
    kFsrTail = 3,   // FSRCNNX<8>'s last layer: prelu(1x1(prelu(conv + b)) + b1 + feat)
};

constexpr int kMaxImg = 16;  // images per launch (the frames of a batch)

// One image of a launch: its maps ([h][w] pixels of 8 16-bit channels) and
// its tiles' place in the launch's tile sequence.
struct ConvImg
{
    const uint4* in;
    uint4* out;
    const uint4* skip;
    const uint4* feat;
    int w, h, tiles_x, tile0;
};

struct ConvParams
{
    const uint4* bw;  // packed B (12 chunks of 256 bytes)
    float b[8], a[8];
    float k1[64], b1[8], a1[8];
    int* status;
    int nimg;
    ConvImg img[kMaxImg];
};

template <bool BF16>
__device__ __forceinline__ void unpack8(const uint4 u, float* v)
{
    const uint32_t r[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        if constexpr (BF16)
        {
            v[2 * i] = __uint_as_float(r[i] << 16);
            v[2 * i + 1] = __uint_as_float(r[i] & 0xFFFF0000u);
        }
        else
        {
            const __half2 h = *reinterpret_cast<const __half2*>(&r[i]);
            const float2 f = __half22float2(h);
            v[2 * i] = f.x;
            v[2 * i + 1] = f.y;
        }
    }
}

template <bool BF16>
__device__ __forceinline__ uint4 pack8(const float* v)
{
    if constexpr (BF16)
        return make_uint4(tc::pack_bf16x2(v[0], v[1]), tc::pack_bf16x2(v[2], v[3]), tc::pack_bf16x2(v[4], v[5]),
                          tc::pack_bf16x2(v[6], v[7]));
    else
        return make_uint4(tc::pack_f16x2(v[0], v[1]), tc::pack_f16x2(v[2], v[3]), tc::pack_f16x2(v[4], v[5]),
                          tc::pack_f16x2(v[6], v[7]));
}

__device__ __forceinline__ float prelu(float v, float a) { return fmaxf(v, 0.0f) + a * fminf(v, 0.0f); }

template <int MODE, bool BF16>
__global__ void __launch_bounds__(THREADS, 4) conv_kernel(const __grid_constant__ ConvParams P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* plane = smem;  // E plane, then O plane
    unsigned char* bsm = smem + 2 * PLANE_BYTES;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(smem + 2 * PLANE_BYTES + B_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + 2 * PLANE_BYTES + B_BYTES + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int im = 0;
    while (im + 1 < P.nimg && P.img[im + 1].tile0 <= static_cast<int>(blockIdx.x)) im++;
    const ConvImg& I = P.img[im];
    const int local = static_cast<int>(blockIdx.x) - I.tile0;
    const int x0 = (local % I.tiles_x) * TW - 1, y0 = (local / I.tiles_x) * TH - 1;

    if (tid == 0)
    {
        tc::mbar_init(mbar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0)
    {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    // weights and the 64x32 window (clamped to the map), loads batched per
    // thread.  The planes' pad slots are zeroed: the first and last valid
    // rows' MMAs read some of them with a zero weight, and a left-over
    // non-finite bit pattern would turn 0 x Inf into NaN.
    for (int i = tid; i < B_BYTES / 16; i += THREADS) reinterpret_cast<uint4*>(bsm)[i] = P.bw[i];
    for (int i = tid; i < 4 * PADP; i += THREADS)
    {
        const int pl = i / (2 * PADP), k = i % (2 * PADP);
        reinterpret_cast<uint4*>(plane + pl * PLANE_BYTES)[k < PADP ? k : NBLK * 128 + k] = make_uint4(0, 0, 0, 0);
    }
    constexpr int PER = WW * WH / THREADS;  // 16
#pragma unroll
    for (int k0 = 0; k0 < PER; k0 += 8)
    {
        uint4 px[8];
#pragma unroll
        for (int k = 0; k < 8; k++)
        {
            const int p = tid + (k0 + k) * THREADS;
            const int wy = p / WW, wx = p - wy * WW;
            const int gx = clampi(x0 + wx, 0, I.w - 1), gy = clampi(y0 + wy, 0, I.h - 1);
            px[k] = I.in[static_cast<size_t>(gy) * I.w + gx];
        }
#pragma unroll
        for (int k = 0; k < 8; k++)
        {
            const int p = tid + (k0 + k) * THREADS;
            reinterpret_cast<uint4*>(plane + ((p & 1) ? PLANE_BYTES : 0))[PADP + (p >> 1)] = px[k];
        }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    if (tid == 0)
    {
        constexpr uint32_t IDESC = tc::idesc_f16(128, 16, BF16);
        const uint64_t a_desc0 = tc::smem_desc(tc::smem_u32(plane) + (PADP - PPR) * 16, PLANE_BYTES - 16, 128);
        const uint64_t b_desc0 = tc::smem_desc(tc::smem_u32(bsm), 256, 128);
        for (int b = 0; b < NBLK; b++)
        {
            const uint64_t a_desc = a_desc0 + static_cast<uint64_t>(b * 128);
#pragma unroll
            for (int dy = 0; dy < 3; dy++)
#pragma unroll
                for (int h = 0; h < 2; h++)
                    tc::mma_f16(tmem + static_cast<uint32_t>(b * 16), a_desc + static_cast<uint64_t>(dy * PPR + h),
                                b_desc0 + static_cast<uint64_t>((2 * dy + h) * 32), IDESC, (dy | h) ? 1u : 0u);
        }
        tc::mma_commit(mbar);
    }
    __syncwarp();
    const bool ok = __syncthreads_and(tc::mbar_wait_ns(mbar, 0, kWaitNs) ? 1 : 0) != 0;
    tc::fence_after_sync();
    if (!ok)
    {
        if (tid == 0) atomicExch(P.status, 1);
    }
    else
        for (int b = 0; b < NBLK; b++)
        {
            float v[16];
            tc::tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(b * 16), v);
            tc::tmem_wait_ld();
            const int r = b * 128 + warp * 32 + lane;
#pragma unroll
            for (int k = 0; k < 2; k++)
            {
                const int p = 2 * r + k;
                const int y = p / WW, x = p - y * WW;
                const int gx = x0 + x, gy = y0 + y;
                if (y < 1 || y > TH || x < 1 || x > TW || gx >= I.w || gy >= I.h) continue;
                const size_t o = static_cast<size_t>(gy) * I.w + gx;
                float s[8];
#pragma unroll
                for (int c = 0; c < 8; c++) s[c] = v[8 * k + c] + P.b[c];
                if constexpr (MODE == kPReLU)
                {
#pragma unroll
                    for (int c = 0; c < 8; c++) s[c] = prelu(s[c], P.a[c]);
                }
                else
                {
                    float sk[8];
                    unpack8<BF16>(I.skip[o], sk);
#pragma unroll
                    for (int c = 0; c < 8; c++) s[c] = fmaf(s[c], 0.2f, sk[c]);
                    if constexpr (MODE == kTail)
                    {
                        float f[8], t[8];
                        unpack8<BF16>(I.feat[o], f);
#pragma unroll
                        for (int n = 0; n < 8; n++)
                        {
                            float u = P.b1[n];
#pragma unroll
                            for (int c = 0; c < 8; c++) u = fmaf(s[c], P.k1[n * 8 + c], u);
                            t[n] = prelu(u, P.a1[n]) + f[n];
                        }
#pragma unroll
                        for (int n = 0; n < 8; n++) s[n] = t[n];
                    }
                }
                I.out[o] = pack8<BF16>(s);
            }
        }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

// Two layers per launch (a residual block of ARNet<8>, or two ACNet<8>
// layers): layer A = conv + PReLU over the whole 64x32 window, drained in
// place into the shared-memory planes once all its MMAs completed (with the
// clamp-to-edge replicas at image borders); layer B = conv + MODE on the
// 60x28 tile, the residual skip being layer A's input map.  Map traffic per
// block: one window read, one skip read, one write (two layers apart: two
// reads, a skip read and two writes).
constexpr int TW2 = WW - 4, TH2 = WH - 4;  // 60 x 28 tile, window origin 2 pixels up and left

struct Conv2Params
{
    const uint4* bwA;  // packed B of layer A
    const uint4* bwB;  // packed B of layer B
    float bA[8], aA[8];
    float b[8], a[8];  // layer B (a: PReLU mode)
    float k1[64], b1[8], a1[8];
    int* status;
    int nimg;
    ConvImg img[kMaxImg];  // in: layer A's input (the skip), out, feat; tiles of TW2 x TH2
};

template <int MODE, bool BF16>
__global__ void __launch_bounds__(THREADS, 4) conv2_kernel(const __grid_constant__ Conv2Params P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* plane = smem;  // E plane, then O plane
    unsigned char* bsmA = smem + 2 * PLANE_BYTES;
    unsigned char* bsmB = bsmA + B_BYTES;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(bsmB + B_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bsmB + B_BYTES + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int im = 0;
    while (im + 1 < P.nimg && P.img[im + 1].tile0 <= static_cast<int>(blockIdx.x)) im++;
    const ConvImg& I = P.img[im];
    const int local = static_cast<int>(blockIdx.x) - I.tile0;
    const int x0 = (local % I.tiles_x) * TW2 - 2, y0 = (local / I.tiles_x) * TH2 - 2;
    // the window's in-image extent
    const int ix0 = max(0, -x0), ix1 = min(WW - 1, I.w - 1 - x0);
    const int iy0 = max(0, -y0), iy1 = min(WH - 1, I.h - 1 - y0);
    const bool edges = ix0 > 0 || ix1 < WW - 1 || iy0 > 0 || iy1 < WH - 1;

    if (tid == 0)
    {
        tc::mbar_init(mbar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0)
    {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    for (int i = tid; i < B_BYTES / 16; i += THREADS)
    {
        reinterpret_cast<uint4*>(bsmA)[i] = P.bwA[i];
        reinterpret_cast<uint4*>(bsmB)[i] = P.bwB[i];
    }
    for (int i = tid; i < 4 * PADP; i += THREADS)
    {
        const int pl = i / (2 * PADP), k = i % (2 * PADP);
        reinterpret_cast<uint4*>(plane + pl * PLANE_BYTES)[k < PADP ? k : NBLK * 128 + k] = make_uint4(0, 0, 0, 0);
    }
    constexpr int PER = WW * WH / THREADS;  // 16
#pragma unroll
    for (int k0 = 0; k0 < PER; k0 += 8)
    {
        uint4 px[8];
#pragma unroll
        for (int k = 0; k < 8; k++)
        {
            const int p = tid + (k0 + k) * THREADS;
            const int wy = p / WW, wx = p - wy * WW;
            const int gx = clampi(x0 + wx, 0, I.w - 1), gy = clampi(y0 + wy, 0, I.h - 1);
            px[k] = I.in[static_cast<size_t>(gy) * I.w + gx];
        }
#pragma unroll
        for (int k = 0; k < 8; k++)
        {
            const int p = tid + (k0 + k) * THREADS;
            reinterpret_cast<uint4*>(plane + ((p & 1) ? PLANE_BYTES : 0))[PADP + (p >> 1)] = px[k];
        }
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t IDESC = tc::idesc_f16(128, 16, BF16);
    const uint64_t a_desc0 = tc::smem_desc(tc::smem_u32(plane) + (PADP - PPR) * 16, PLANE_BYTES - 16, 128);

    bool ok = true;
#pragma unroll 1
    for (int layer = 0; layer < 2; layer++)
    {
        if (tid == 0)
        {
            const uint64_t b_desc0 = tc::smem_desc(tc::smem_u32(layer ? bsmB : bsmA), 256, 128);
            for (int b = 0; b < NBLK; b++)
            {
                const uint64_t a_desc = a_desc0 + static_cast<uint64_t>(b * 128);
#pragma unroll
                for (int dy = 0; dy < 3; dy++)
#pragma unroll
                    for (int h = 0; h < 2; h++)
                        tc::mma_f16(tmem + static_cast<uint32_t>(b * 16), a_desc + static_cast<uint64_t>(dy * PPR + h),
                                    b_desc0 + static_cast<uint64_t>((2 * dy + h) * 32), IDESC, (dy | h) ? 1u : 0u);
            }
            tc::mma_commit(mbar);
        }
        __syncwarp();
        ok = __syncthreads_and((ok && tc::mbar_wait_ns(mbar, static_cast<uint32_t>(layer), kWaitNs)) ? 1 : 0) != 0;
        tc::fence_after_sync();
        if (!ok)
        {
            if (tid == 0) atomicExch(P.status, 1);
            break;
        }
        if (layer == 0)
        {
            // layer A: prelu(conv + b) for window pixels 1 .. W-2 inside the image, in place
            const int ry0 = max(1, iy0), ry1 = min(WH - 2, iy1), rx0 = max(1, ix0), rx1 = min(WW - 2, ix1);
            for (int b = 0; b < NBLK; b++)
            {
                float v[16];
                tc::tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(b * 16), v);
                tc::tmem_wait_ld();
                const int r = b * 128 + warp * 32 + lane;
#pragma unroll
                for (int k = 0; k < 2; k++)
                {
                    const int p = 2 * r + k;
                    const int y = p / WW, x = p - y * WW;
                    if (y < ry0 || y > ry1 || x < rx0 || x > rx1) continue;
                    float sv[8];
#pragma unroll
                    for (int c = 0; c < 8; c++) sv[c] = prelu(v[8 * k + c] + P.bA[c], P.aA[c]);
                    const uint4 val = pack8<BF16>(sv);
                    auto put = [&](int q) {
                        reinterpret_cast<uint4*>(plane + ((q & 1) ? PLANE_BYTES : 0))[PADP + (q >> 1)] = val;
                    };
                    put(p);
                    // clamp-to-edge for layer B (only tiles at an image edge)
                    if (!edges) continue;
                    const bool xl = x == ix0 && x > 0, xr = x == ix1 && x < WW - 1;
                    const bool yt = y == iy0 && y > 0, yb = y == iy1 && y < WH - 1;
                    if (xl) put(p - 1);
                    if (xr) put(p + 1);
                    if (yt)
                    {
                        put(p - WW);
                        if (xl) put(p - WW - 1);
                        if (xr) put(p - WW + 1);
                    }
                    if (yb)
                    {
                        put(p + WW);
                        if (xl) put(p + WW - 1);
                        if (xr) put(p + WW + 1);
                    }
                }
            }
            tc::fence_proxy_async_smem();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
        else
        {
            // layer B on the tile: window pixels 2 .. W-3 inside the image
            for (int b = 0; b < NBLK; b++)
            {
                float v[16];
                tc::tmem_ld16(tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(b * 16), v);
                tc::tmem_wait_ld();
                const int r = b * 128 + warp * 32 + lane;
#pragma unroll
                for (int k = 0; k < 2; k++)
                {
                    const int p = 2 * r + k;
                    const int y = p / WW, x = p - y * WW;
                    const int gx = x0 + x, gy = y0 + y;
                    if (y < 2 || y > WH - 3 || x < 2 || x > WW - 3 || gx >= I.w || gy >= I.h) continue;
                    const size_t o = static_cast<size_t>(gy) * I.w + gx;
                    float sv[8];
#pragma unroll
                    for (int c = 0; c < 8; c++) sv[c] = v[8 * k + c] + P.b[c];
                    if constexpr (MODE == kPReLU)
                    {
#pragma unroll
                        for (int c = 0; c < 8; c++) sv[c] = prelu(sv[c], P.a[c]);
                    }
                    else if constexpr (MODE == kFsrTail)
                    {
                        // conv3x3 + PReLU, conv1x1 8->8 + bias + feat, PReLU
                        // (CPUProcessor.cpp:1629-1715 order, as k_f3_fp32.cu's tail)
                        float f[8], t[8];
                        unpack8<BF16>(I.feat[o], f);
#pragma unroll
                        for (int c = 0; c < 8; c++) sv[c] = prelu(sv[c], P.a[c]);
#pragma unroll
                        for (int n = 0; n < 8; n++)
                        {
                            float u = P.b1[n];
#pragma unroll
                            for (int c = 0; c < 8; c++) u = fmaf(sv[c], P.k1[n * 8 + c], u);
                            t[n] = prelu(u + f[n], P.a1[n]);
                        }
#pragma unroll
                        for (int n = 0; n < 8; n++) sv[n] = t[n];
                    }
                    else
                    {
                        float sk[8];
                        unpack8<BF16>(I.in[o], sk);
#pragma unroll
                        for (int c = 0; c < 8; c++) sv[c] = fmaf(sv[c], 0.2f, sk[c]);
                        if constexpr (MODE == kTail)
                        {
                            float f[8], t[8];
                            unpack8<BF16>(I.feat[o], f);
#pragma unroll
                            for (int n = 0; n < 8; n++)
                            {
                                float u = P.b1[n];
#pragma unroll
                                for (int c = 0; c < 8; c++) u = fmaf(sv[c], P.k1[n * 8 + c], u);
                                t[n] = prelu(u, P.a1[n]) + f[n];
                            }
#pragma unroll
                            for (int n = 0; n < 8; n++) sv[n] = t[n];
                        }
                    }
                    I.out[o] = pack8<BF16>(sv);
                }
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

struct HeadParams
{
    float k[72];
    unsigned long long kd[72];  // each weight twice, (k, k), for the paired FMAs (filled by launch_head)
    float b[8];
    float a[8];   // PReLU slopes when `prelu` is set (the ACNet<8> head)
    int prelu;
    Plane in[kMaxImg];     // image blockIdx.z
    uint4* feat[kMaxImg];
};

// Head: conv3x3 1->8 in FP32 from the input plane, identity (ARNet) or PReLU
// (ACNet<8>), stored as a 16-bit 8-channel map, taps clamped to the plane:
// head2_kernel below.

struct UpParams
{
    float k[288];
    unsigned long long kd[288];  // each weight twice, (k, k): an operand of the paired FMAs (filled by launch_up)
    float b[4];
    int no_nearest;  // FSRCNNX<8>: no nearest-input add
    const uint4* map[kMaxImg];  // image blockIdx.z
    Plane src[kMaxImg], dst[kMaxImg];
};

// Two FP32 lanes in a 64-bit register pair and the paired fused
// multiply-add (fma.rn.f32x2): each lane is exactly fmaf.
__device__ __forceinline__ unsigned long long pk2(float lo, float hi)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void upk2(unsigned long long v, float& lo, float& hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Upscale: conv3x3 8->4 (identity) in FP32 from the 16-bit map, pixel
// shuffle 2x2, plus the nearest input pixel, fromFloat (Common.hpp:290-342).
// Two horizontally adjacent pixels per thread, in the lanes of paired FMAs:
// each output is the fmaf chain over the taps (rows, columns, channels in
// that order) from the bias; the pair shares its taps' middle columns (four
// map columns per row instead of six).
template <typename T, bool BF16>
__global__ void __launch_bounds__(256) up2_kernel(const __grid_constant__ UpParams U)
{
    const uint4* __restrict__ map = U.map[blockIdx.z];
    const Plane& src = U.src[blockIdx.z];
    const Plane& dst = U.dst[blockIdx.z];
    const int w = src.w, h = src.h;
    const int x = 2 * (blockIdx.x * 32 + (threadIdx.x & 31)), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= w || y >= h) return;
    const bool has_b = x + 1 < w;
    unsigned long long acc[4];
#pragma unroll
    for (int n = 0; n < 4; n++) acc[n] = pk2(U.b[n], U.b[n]);
#pragma unroll
    for (int dy = 0; dy < 3; dy++)
    {
        const int gy = clampi(y + dy - 1, 0, h - 1);
        float xv[4][8];  // map columns x - 1 .. x + 2 (clamped)
#pragma unroll
        for (int j = 0; j < 4; j++) unpack8<BF16>(map[static_cast<size_t>(gy) * w + clampi(x - 1 + j, 0, w - 1)], xv[j]);
#pragma unroll
        for (int dx = 0; dx < 3; dx++)
#pragma unroll
            for (int c = 0; c < 8; c++)
            {
                const unsigned long long xp = pk2(xv[dx][c], xv[dx + 1][c]);  // (pixel x, pixel x + 1)
#pragma unroll
                for (int n = 0; n < 4; n++) acc[n] = fma2(xp, U.kd[n * 72 + (dy * 3 + dx) * 8 + c], acc[n]);
            }
    }
    const T* srow = row_ptr<T>(src.ptr, src.pitch, y);
    const float near_a = U.no_nearest ? 0.0f : to_float<T>(srow[x]);
    const float near_b = U.no_nearest || !has_b ? 0.0f : to_float<T>(srow[x + 1]);
#pragma unroll
    for (int n = 0; n < 4; n++)
    {
        float a, b;
        upk2(acc[n], a, b);
        T* orow = row_ptr_w<T>(dst.ptr, dst.pitch, 2 * y + (n >> 1));
        orow[2 * x + (n & 1)] = from_float<T>(a + near_a);
        if (has_b) orow[2 * x + 2 + (n & 1)] = from_float<T>(b + near_b);
    }
}

// The head, two horizontally adjacent pixels per thread in the lanes of
// paired FMAs: each output is the fmaf chain over the nine taps from the
// bias; the pair shares its taps' middle columns.
template <typename T, bool BF16>
__global__ void __launch_bounds__(256) head2_kernel(const __grid_constant__ HeadParams P)
{
    const Plane& in = P.in[blockIdx.z];
    uint4* __restrict__ feat = P.feat[blockIdx.z];
    const int x = 2 * (blockIdx.x * 32 + (threadIdx.x & 31)), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= in.w || y >= in.h) return;
    const bool has_b = x + 1 < in.w;
    unsigned long long t[9];  // tap p of (pixel x, pixel x + 1)
#pragma unroll
    for (int dy = 0; dy < 3; dy++)
    {
        const T* row = row_ptr<T>(in.ptr, in.pitch, clampi(y + dy - 1, 0, in.h - 1));
        float c4[4];  // columns x - 1 .. x + 2 (clamped)
#pragma unroll
        for (int j = 0; j < 4; j++) c4[j] = to_float<T>(row[clampi(x - 1 + j, 0, in.w - 1)]);
#pragma unroll
        for (int dx = 0; dx < 3; dx++) t[dy * 3 + dx] = pk2(c4[dx], c4[dx + 1]);
    }
    float ra[8], rb[8];
#pragma unroll
    for (int n = 0; n < 8; n++)
    {
        unsigned long long v = pk2(P.b[n], P.b[n]);
#pragma unroll
        for (int p = 0; p < 9; p++) v = fma2(t[p], P.kd[n * 9 + p], v);
        float a, b;
        upk2(v, a, b);
        ra[n] = P.prelu ? prelu(a, P.a[n]) : a;
        rb[n] = P.prelu ? prelu(b, P.a[n]) : b;
    }
    feat[static_cast<size_t>(y) * in.w + x] = pack8<BF16>(ra);
    if (has_b) feat[static_cast<size_t>(y) * in.w + x + 1] = pack8<BF16>(rb);
}

template <int MODE, bool BF16>
cudaError_t launch_conv(const ConvParams& p, int tiles, cudaStream_t stream)
{
    // one-time set-up per device, thread-safe
    const cudaError_t setup = device_once([] {
        return cudaFuncSetAttribute(conv_kernel<MODE, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_REQ);
    });
    if (setup != cudaSuccess) return setup;
    conv_kernel<MODE, BF16><<<tiles, THREADS, SMEM_REQ, stream>>>(p);
    return cudaGetLastError();
}

constexpr int SMEM2 = 2 * PLANE_BYTES + 2 * B_BYTES + 64;
constexpr int SMEM2_REQ = SMEM2 > 48 * 1024 ? SMEM2 : 48 * 1024;  // at most four CTAs per SM (tensor memory)

template <int MODE, bool BF16>
cudaError_t launch_conv2(const Conv2Params& p, int tiles, cudaStream_t stream)
{
    // one-time set-up per device, thread-safe
    const cudaError_t setup = device_once([] {
        return cudaFuncSetAttribute(conv2_kernel<MODE, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM2_REQ);
    });
    if (setup != cudaSuccess) return setup;
    conv2_kernel<MODE, BF16><<<tiles, THREADS, SMEM2_REQ, stream>>>(p);
    return cudaGetLastError();
}

uint16_t to_bits(float v, bool bf16)
{
    if (bf16)
    {
        uint32_t u;
        std::memcpy(&u, &v, 4);
        return static_cast<uint16_t>((u + 0x7FFFu + ((u >> 16) & 1u)) >> 16);
    }
    return __half_as_ushort(__float2half_rn(v));
}

}  // namespace arnettc

// Packs the 3x3 8->8 kernel k[n*72 + tap*8 + c] of one layer for the pair
// formulation: chunk j (0..11) of 256 bytes, output column n (0..15; n < 8 is
// pixel 2r, n >= 8 pixel 2r+1, channel n % 8), input channel c.  MMA 2*dy
// multiplies chunks 4dy (even pixel r+s) and 4dy+1 (odd pixel r-1+s), MMA
// 2dy+1 chunks 4dy+2 (even r+1+s) and 4dy+3 (odd r+s); for pixel 2r the taps
// dx = 0, 1, 2 sit at odd r-1, even r, odd r; for pixel 2r+1 at even r, odd r,
// even r+1.
void pack_pair_conv8(const float* k, bool bf16, uint16_t* out)
{
    using arnettc::to_bits;
    std::memset(out, 0, 12 * 256);
    auto put = [&](int chunk, int n, int dx, int dy) {
        for (int c = 0; c < 8; c++) out[(chunk * 256 + (n / 8) * 128 + (n % 8) * 16) / 2 + c] = to_bits(k[(n % 8) * 72 + (dy * 3 + dx) * 8 + c], bf16);
    };
    for (int dy = 0; dy < 3; dy++)
        for (int n = 0; n < 16; n++)
        {
            const bool odd = n >= 8;
            put(4 * dy + 0, n, odd ? 0 : 1, dy);      // even pixel r
            if (!odd) put(4 * dy + 1, n, 0, dy);      // odd pixel r-1
            if (odd) put(4 * dy + 2, n, 2, dy);       // even pixel r+1
            put(4 * dy + 3, n, odd ? 1 : 2, dy);      // odd pixel r
        }
}

namespace arnettc {

// The head over n images (grid z = image); hp.in / hp.feat filled in.
cudaError_t launch_head(const HeadParams& hp0, bool bf16, int n, cudaStream_t stream)
{
    HeadParams hp = hp0;
    for (int i = 0; i < 72; i++)
    {
        unsigned int b;
        std::memcpy(&b, &hp.k[i], 4);
        hp.kd[i] = (static_cast<unsigned long long>(b) << 32) | b;
    }
    int mw = 0, mh = 0;
    for (int i = 0; i < n; i++)
    {
        mw = hp.in[i].w > mw ? hp.in[i].w : mw;
        mh = hp.in[i].h > mh ? hp.in[i].h : mh;
    }
    // two pixels per thread
    const dim3 pgrid((mw + 63) / 64, (mh + 7) / 8, n);
    switch (hp.in[0].type)
    {
    case kU8: bf16 ? head2_kernel<uint8_t, true><<<pgrid, 256, 0, stream>>>(hp) : head2_kernel<uint8_t, false><<<pgrid, 256, 0, stream>>>(hp); break;
    case kU16: bf16 ? head2_kernel<uint16_t, true><<<pgrid, 256, 0, stream>>>(hp) : head2_kernel<uint16_t, false><<<pgrid, 256, 0, stream>>>(hp); break;
    case kF32: bf16 ? head2_kernel<float, true><<<pgrid, 256, 0, stream>>>(hp) : head2_kernel<float, false><<<pgrid, 256, 0, stream>>>(hp); break;
    default: return cudaErrorInvalidValue;
    }
    const cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) count_launch();
    return err;
}

// The upscale layer over n images (grid z = image); u.map / src / dst filled in.
cudaError_t launch_up(const UpParams& u0, bool bf16, int n, cudaStream_t stream)
{
    UpParams u = u0;
    for (int i = 0; i < 288; i++)
    {
        unsigned int b;
        std::memcpy(&b, &u.k[i], 4);
        u.kd[i] = (static_cast<unsigned long long>(b) << 32) | b;
    }
    int mw = 0, mh = 0;
    for (int i = 0; i < n; i++)
    {
        mw = u.src[i].w > mw ? u.src[i].w : mw;
        mh = u.src[i].h > mh ? u.src[i].h : mh;
    }
    // two pixels per thread
    const dim3 pgrid((mw + 63) / 64, (mh + 7) / 8, n);
    switch (u.src[0].type)
    {
    case kU8: bf16 ? up2_kernel<uint8_t, true><<<pgrid, 256, 0, stream>>>(u) : up2_kernel<uint8_t, false><<<pgrid, 256, 0, stream>>>(u); break;
    case kU16: bf16 ? up2_kernel<uint16_t, true><<<pgrid, 256, 0, stream>>>(u) : up2_kernel<uint16_t, false><<<pgrid, 256, 0, stream>>>(u); break;
    case kF32: bf16 ? up2_kernel<float, true><<<pgrid, 256, 0, stream>>>(u) : up2_kernel<float, false><<<pgrid, 256, 0, stream>>>(u); break;
    default: return cudaErrorInvalidValue;
    }
    const cudaError_t err = cudaGetLastError();
    if (err == cudaSuccess) count_launch();
    return err;
}

// Checks a batch (1 to kMaxImg single-channel images of one element type,
// each output 2x its input) and fills the per-image parts of the launch
// parameters: tile sequence of the conv launches, head and upscale planes.
cudaError_t prepare_batch(int n, const Plane* in, const Plane* out, ConvParams& c, HeadParams& hp, UpParams& u, int& tiles)
{
    if (n < 1 || n > kMaxImg) return cudaErrorInvalidValue;
    tiles = 0;
    for (int i = 0; i < n; i++)
    {
        if (in[i].w <= 0 || in[i].h <= 0 || in[i].channels != 1 || out[i].channels != 1 || in[i].type != in[0].type ||
            out[i].w != 2 * in[i].w || out[i].h != 2 * in[i].h)
            return cudaErrorInvalidValue;
        ConvImg& I = c.img[i];
        I.w = in[i].w;
        I.h = in[i].h;
        I.tiles_x = (in[i].w + TW - 1) / TW;
        I.tile0 = tiles;
        tiles += I.tiles_x * ((in[i].h + TH - 1) / TH);
        hp.in[i] = in[i];
        u.src[i] = in[i];
        u.dst[i] = out[i];
    }
    c.nimg = n;
    return cudaSuccess;
}

// Tiles of the two-layer launches (TW2 x TH2) for the images of a prepared batch.
int fill_tiles2(int n, const ConvParams& c, Conv2Params& c2)
{
    int tiles = 0;
    for (int i = 0; i < n; i++)
    {
        ConvImg& I = c2.img[i];
        I.w = c.img[i].w;
        I.h = c.img[i].h;
        I.tiles_x = (I.w + TW2 - 1) / TW2;
        I.tile0 = tiles;
        tiles += I.tiles_x * ((I.h + TH2 - 1) / TH2);
    }
    c2.nimg = n;
    return tiles;
}

}  // namespace arnettc

// Runs one ARNet x2 pass over n images in the tensor-core form, every layer
// as one launch over all images.  packed: 2*blocks layers of pack_pair_conv8
// output (device); maps[3 i + j]: image i's three [h][w] arrays of 16-byte
// pixels.
cudaError_t launch_arnet_tc_batch(const float* kernels, const float* biases, const float* alphas, int blocks, const void* packed,
                                  bool bf16, int n, const Plane* in, const Plane* out, void* const* maps, int* status,
                                  cudaStream_t stream)
{
    using namespace arnettc;
    if (n <= 0) return cudaSuccess;
    if (blocks < 2 || !packed || !status || !maps) return cudaErrorInvalidValue;
    ConvParams p;
    HeadParams hp;
    UpParams u;
    std::memset(&p, 0, sizeof(p));
    std::memset(&hp, 0, sizeof(hp));
    std::memset(&u, 0, sizeof(u));
    int tiles = 0;
    cudaError_t err = prepare_batch(n, in, out, p, hp, u, tiles);
    if (err != cudaSuccess) return err;
    p.status = status;
    // head (FP32)
    for (int i = 0; i < 72; i++) hp.k[i] = kernels[i];
    for (int i = 0; i < 8; i++) hp.b[i] = biases[i];
    hp.prelu = 0;
    for (int i = 0; i < n; i++) hp.feat[i] = static_cast<uint4*>(maps[3 * i]);
    if ((err = launch_head(hp, bf16, n, stream)) != cudaSuccess) return err;
    // each residual block as one two-layer launch: maps of image i are
    // feat, then two maps used in turn (the block's input and output)
    constexpr int FEAT = 0;
    Conv2Params c2;
    std::memset(&c2, 0, sizeof(c2));
    const int tiles2 = fill_tiles2(n, p, c2);
    c2.status = status;
    int cur = FEAT;
    int l = 1;
    for (int blk = 0; blk < blocks; blk++)
    {
        const bool tail = blk == blocks - 1;
        const int nxt = cur == 1 ? 2 : 1;
        Conv2Params c = c2;
        for (int i = 0; i < n; i++)
        {
            c.img[i].in = static_cast<const uint4*>(maps[3 * i + cur]);
            c.img[i].out = static_cast<uint4*>(maps[3 * i + nxt]);
            c.img[i].feat = static_cast<const uint4*>(maps[3 * i + FEAT]);
        }
        // layer l: conv + PReLU; layer l+1: 0.2 conv + the block input (+ the 1x1 tail)
        c.bwA = static_cast<const uint4*>(packed) + static_cast<size_t>(l - 1) * (B_BYTES / 16);
        c.bwB = static_cast<const uint4*>(packed) + static_cast<size_t>(l) * (B_BYTES / 16);
        for (int i = 0; i < 8; i++) c.bA[i] = biases[8 * l + i];
        for (int i = 0; i < 8; i++) c.aA[i] = alphas[8 * ((l - 1) / 2) + i];
        for (int i = 0; i < 8; i++) c.b[i] = biases[8 * (l + 1) + i];
        if (tail)
        {
            for (int i = 0; i < 64; i++) c.k1[i] = kernels[72 + 576 * (2 * blocks) + i];
            for (int i = 0; i < 8; i++) c.b1[i] = biases[8 * (l + 2) + i];
            for (int i = 0; i < 8; i++) c.a1[i] = alphas[8 * blocks + i];
            err = bf16 ? launch_conv2<kTail, true>(c, tiles2, stream) : launch_conv2<kTail, false>(c, tiles2, stream);
        }
        else err = bf16 ? launch_conv2<kResidual, true>(c, tiles2, stream) : launch_conv2<kResidual, false>(c, tiles2, stream);
        if (err != cudaSuccess) return err;
        count_launch();
        l += 2;
        cur = nxt;
    }
    const int X = cur;  // the last block's output
    l++;  // the 1x1 layer's bias index
    // upscale (FP32)
    for (int i = 0; i < 288; i++) u.k[i] = kernels[72 + 576 * (2 * blocks) + 64 + i];
    for (int i = 0; i < 4; i++) u.b[i] = biases[8 * l + i];
    for (int i = 0; i < n; i++) u.map[i] = static_cast<const uint4*>(maps[3 * i + X]);
    return launch_up(u, bf16, n, stream);
}

cudaError_t launch_arnet_tc(const float* kernels, const float* biases, const float* alphas, int blocks, const void* packed,
                            bool bf16, const Plane& in, const Plane& out, void* const maps[3], int* status,
                            cudaStream_t stream)
{
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    return launch_arnet_tc_batch(kernels, biases, alphas, blocks, packed, bf16, 1, &in, &out, maps, status, stream);
}

// Runs one ACNet<8> x2 pass over n images in the tensor-core form (network of
// core/include/AC/Core/Model/ACNet.hpp:63-116, CPU order
// core/src/processor/cpu/CPUProcessor.cpp:1417-1436): the PReLU head in FP32,
// `blocks` 3x3 8->8 + PReLU layers on tcgen05 (packed: `blocks` layers of
// pack_pair_conv8 output), the upscale layer in FP32.  maps[2 i + j]: image
// i's two [h][w] arrays of 16-byte pixels, used in turn.
cudaError_t launch_acnet8_tc_batch(const float* kernels, const float* biases, const float* alphas, int blocks,
                                   const void* packed, bool bf16, int n, const Plane* in, const Plane* out,
                                   void* const* maps, int* status, cudaStream_t stream)
{
    using namespace arnettc;
    if (n <= 0) return cudaSuccess;
    if (blocks < 1 || !packed || !status || !maps) return cudaErrorInvalidValue;
    ConvParams c;
    HeadParams hp;
    UpParams u;
    std::memset(&c, 0, sizeof(c));
    std::memset(&hp, 0, sizeof(hp));
    std::memset(&u, 0, sizeof(u));
    int tiles = 0;
    cudaError_t err = prepare_batch(n, in, out, c, hp, u, tiles);
    if (err != cudaSuccess) return err;
    c.status = status;
    for (int i = 0; i < 72; i++) hp.k[i] = kernels[i];
    for (int i = 0; i < 8; i++) hp.b[i] = biases[i];
    for (int i = 0; i < 8; i++) hp.a[i] = alphas[i];
    hp.prelu = 1;
    for (int i = 0; i < n; i++) hp.feat[i] = static_cast<uint4*>(maps[2 * i]);
    if ((err = launch_head(hp, bf16, n, stream)) != cudaSuccess) return err;
    int a = 0;  // the map holding the current layer's input
    Conv2Params c2;
    std::memset(&c2, 0, sizeof(c2));
    const int tiles2 = fill_tiles2(n, c, c2);
    c2.status = status;
    int l = 1;
    // pairs of layers as one two-layer launch
    for (; l + 1 <= blocks; l += 2)
    {
        Conv2Params q = c2;
        for (int i = 0; i < n; i++)
        {
            q.img[i].in = static_cast<const uint4*>(maps[2 * i + a]);
            q.img[i].out = static_cast<uint4*>(maps[2 * i + 1 - a]);
        }
        q.bwA = static_cast<const uint4*>(packed) + static_cast<size_t>(l - 1) * (B_BYTES / 16);
        q.bwB = static_cast<const uint4*>(packed) + static_cast<size_t>(l) * (B_BYTES / 16);
        for (int i = 0; i < 8; i++) q.bA[i] = biases[8 * l + i];
        for (int i = 0; i < 8; i++) q.aA[i] = alphas[8 * l + i];
        for (int i = 0; i < 8; i++) q.b[i] = biases[8 * (l + 1) + i];
        for (int i = 0; i < 8; i++) q.a[i] = alphas[8 * (l + 1) + i];
        err = bf16 ? launch_conv2<kPReLU, true>(q, tiles2, stream) : launch_conv2<kPReLU, false>(q, tiles2, stream);
        if (err != cudaSuccess) return err;
        count_launch();
        a = 1 - a;
    }
    // an odd last layer on its own
    if (l == blocks)
    {
        for (int i = 0; i < n; i++)
        {
            c.img[i].in = static_cast<const uint4*>(maps[2 * i + a]);
            c.img[i].out = static_cast<uint4*>(maps[2 * i + 1 - a]);
        }
        c.bw = static_cast<const uint4*>(packed) + static_cast<size_t>(l - 1) * (B_BYTES / 16);
        for (int i = 0; i < 8; i++) c.b[i] = biases[8 * l + i];
        for (int i = 0; i < 8; i++) c.a[i] = alphas[8 * l + i];
        err = bf16 ? launch_conv<kPReLU, true>(c, tiles, stream) : launch_conv<kPReLU, false>(c, tiles, stream);
        if (err != cudaSuccess) return err;
        count_launch();
        a = 1 - a;
    }
    for (int i = 0; i < 288; i++) u.k[i] = kernels[72 + 576 * blocks + i];
    for (int i = 0; i < 4; i++) u.b[i] = biases[8 * (blocks + 1) + i];
    for (int i = 0; i < n; i++) u.map[i] = static_cast<const uint4*>(maps[2 * i + a]);
    return launch_up(u, bf16, n, stream);
}

cudaError_t launch_acnet8_tc(const float* kernels, const float* biases, const float* alphas, int blocks, const void* packed,
                             bool bf16, const Plane& in, const Plane& out, void* const maps[2], int* status,
                             cudaStream_t stream)
{
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    return launch_acnet8_tc_batch(kernels, biases, alphas, blocks, packed, bf16, 1, &in, &out, maps, status, stream);
}

// FSRCNNX<8> (B4) x2 in the tensor-core form over n single-channel images of
// one element type, every layer as one launch over all of them: the 5x5 head
// in FP32 (launch_f3_head8), layers 1 + 2 and 3 + the tail as two two-layer
// launches (the tail: PReLU, conv1x1 8->8 + feat, PReLU), the upscale conv3x3
// 8->4 + pixel shuffle in FP32 without the nearest-input add.  Parameters in
// the reference layout (FSRCNNX.hpp:28-66): kernels head 200, 4 x 576, 1x1 64,
// upscale 288; biases 8 per layer (head, 4 convs, 1x1) then 4; PReLU slopes
// 8 per layer (4 convs, then the one after the 1x1).  packed: the 4 layers'
// pack_pair_conv8 output; maps[3 i + j]: image i's three [h][w] arrays of
// 16-byte pixels.
cudaError_t launch_fsrcnnx8_tc_batch(const float* kernels, const float* biases, const float* alphas, const void* packed, bool bf16,
                                     int n, const Plane* in, const Plane* out, void* const* maps, int* status, cudaStream_t stream)
{
    using namespace arnettc;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxImg || !packed || !status || !maps) return cudaErrorInvalidValue;
    void* feat[kMaxImg];
    Conv2Params c2;
    std::memset(&c2, 0, sizeof(c2));
    int tiles2 = 0;
    for (int i = 0; i < n; i++)
    {
        if (in[i].w <= 0 || in[i].h <= 0 || in[i].channels != 1 || out[i].channels != 1 || in[i].type != in[0].type ||
            out[i].w != 2 * in[i].w || out[i].h != 2 * in[i].h)
            return cudaErrorInvalidValue;
        feat[i] = maps[3 * i];
        ConvImg& I = c2.img[i];
        I.w = in[i].w;
        I.h = in[i].h;
        I.tiles_x = (in[i].w + TW2 - 1) / TW2;
        I.tile0 = tiles2;
        I.feat = static_cast<const uint4*>(maps[3 * i]);
        tiles2 += I.tiles_x * ((in[i].h + TH2 - 1) / TH2);
    }
    c2.nimg = n;
    c2.status = status;
    cudaError_t err = launch_f3_head8(kernels, biases, bf16, n, in, feat, stream);
    if (err != cudaSuccess) return err;
    count_launch();
    const uint4* pk = static_cast<const uint4*>(packed);
    // layers 1 and 2 (PReLU): map 0 -> map 1
    {
        Conv2Params q = c2;
        for (int i = 0; i < n; i++)
        {
            q.img[i].in = static_cast<const uint4*>(maps[3 * i]);
            q.img[i].out = static_cast<uint4*>(maps[3 * i + 1]);
        }
        q.bwA = pk;
        q.bwB = pk + (B_BYTES / 16);
        for (int i = 0; i < 8; i++)
        {
            q.bA[i] = biases[8 + i];
            q.aA[i] = alphas[i];
            q.b[i] = biases[16 + i];
            q.a[i] = alphas[8 + i];
        }
        err = bf16 ? launch_conv2<kPReLU, true>(q, tiles2, stream) : launch_conv2<kPReLU, false>(q, tiles2, stream);
        if (err != cudaSuccess) return err;
        count_launch();
    }
    // layer 3 (PReLU) and the tail: map 1 -> map 2
    {
        Conv2Params q = c2;
        for (int i = 0; i < n; i++)
        {
            q.img[i].in = static_cast<const uint4*>(maps[3 * i + 1]);
            q.img[i].out = static_cast<uint4*>(maps[3 * i + 2]);
        }
        q.bwA = pk + 2 * (B_BYTES / 16);
        q.bwB = pk + 3 * (B_BYTES / 16);
        for (int i = 0; i < 8; i++)
        {
            q.bA[i] = biases[24 + i];
            q.aA[i] = alphas[16 + i];
            q.b[i] = biases[32 + i];
            q.a[i] = alphas[24 + i];
            q.b1[i] = biases[40 + i];
            q.a1[i] = alphas[32 + i];
        }
        for (int i = 0; i < 64; i++) q.k1[i] = kernels[200 + 4 * 576 + i];
        err = bf16 ? launch_conv2<kFsrTail, true>(q, tiles2, stream) : launch_conv2<kFsrTail, false>(q, tiles2, stream);
        if (err != cudaSuccess) return err;
        count_launch();
    }
    UpParams u;
    std::memset(&u, 0, sizeof(u));
    for (int i = 0; i < 288; i++) u.k[i] = kernels[200 + 4 * 576 + 64 + i];
    for (int i = 0; i < 4; i++) u.b[i] = biases[48 + i];
    u.no_nearest = 1;
    for (int i = 0; i < n; i++)
    {
        u.map[i] = static_cast<const uint4*>(maps[3 * i + 2]);
        u.src[i] = in[i];
        u.dst[i] = out[i];
    }
    return launch_up(u, bf16, n, stream);
}

cudaError_t launch_fsrcnnx8_tc(const float* kernels, const float* biases, const float* alphas, const void* packed, bool bf16,
                               const Plane& in, const Plane& out, void* const maps[3], int* status, cudaStream_t stream)
{
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    return launch_fsrcnnx8_tc_batch(kernels, biases, alphas, packed, bf16, 1, &in, &out, maps, status, stream);
}

}  // namespace acgb
