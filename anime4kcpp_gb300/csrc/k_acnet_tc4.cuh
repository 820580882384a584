#pragma once
// Persistent, warp-specialised tensor-core ACNetLegacy x2 kernel with four
// pixels per GEMM row (quad formulation).
//
// Network, clamp semantics, fused colour, tile queue, bias-in-accumulator
// and bounded waits are those of the pair kernel (k_acnet_tc3.cuh; reference
// layer math core/internal/AC/Core/Internal/Processor/CPU/Common.hpp:116-197,
// 344-393).  What changes is the GEMM shape:
//
//  * One GEMM row = four horizontally adjacent pixels 4r .. 4r+3 of the
//    window, N = 4 x 8 output channels = 32.  Activations live as four planes
//    (pixel index mod 4), 16 bytes (8 FP16/BF16 channels) per pixel.  A tap
//    row needs the six pixels 4r-1 .. 4r+4, read as three K16 chunks whose
//    two 8-channel halves come from two planes: (P0[r], P3[r-1]),
//    (P1[r], P2[r]), (P0[r+1], P3[r]); the first and third share one
//    descriptor form (leading byte offset 3 planes - 16 bytes), the second
//    has offset 1 plane.  Nine M128 x N32 x K16 MMAs per 128 rows and layer:
//    512 pixels, against twelve M128 x N16 x K16 MMAs for the same pixels in
//    the pair form.  Each MMA costs about the same (its 4 KB A operand is
//    read from shared memory), so a layer takes 25 % less tensor-core time.
//  * A window of 64 x 64 pixels (halo 9 around a 46 x 46 tile) is 8 blocks of
//    128 rows, 32 tensor-memory columns each (256 per CTA, two CTAs per SM).
//    Four rounds of two blocks per layer; MMA warp i issues block 2r + i of
//    round r, epilogue group g drains block 2r + g.
//  * A layer's B matrices (9 KB) stream through a three-slot ring in shared
//    memory: the first MMA warp bulk-copies layer G + 2 (counting layers over
//    the CTA's tiles) into the slot of layer G - 1 once every MMA of layer
//    G - 1 completed, so the weights of all nine layers never sit in shared
//    memory at once and two CTAs still share an SM.
//
// The same kernel runs ACNet<8> with 4 or 8 blocks (NetAcn8; reference
// CPUProcessor.cpp:1417-1436, Common.hpp:290-342): layer 0 and the blocks
// with PReLU (per layer and channel slopes) instead of ReLU, and as its last
// MMA layer the conv3x3 8 -> 4 (channels 4..7 carry the 16-bit residuals of
// the weights of channels 0..3, summed in the epilogue) whose outputs are
// pixel-shuffled and added to the source pixel (nearest) instead of
// ACNetLegacy's 2x2 transposed conv.  The halo is the number of 3x3
// layers: 9 (ACNetLegacy), 6 (ACNet<8> B4), 10 (B8).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

#include "colour.cuh"
#include "device_common.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"
#include "tma_host.hpp"

namespace acgb {
namespace tcv4 {

constexpr int NBLK = 8;                      // 8 x 128 quad rows per window
constexpr int NROUND = 4;                    // two blocks (one per issuer) per round
constexpr int KCH = 9;                       // MMAs (K16 chunks) per block and layer
constexpr int CHUNK_BYTES = 1024;            // B of one MMA: N32 x K16 x 16 bit
constexpr int BL_BYTES = KCH * CHUNK_BYTES;  // one layer's B
constexpr int NLMAX = 10;  // MMA layers of the deepest network run here (ACNet<8> B8)
constexpr int NBUF = 3;                      // B ring slots
constexpr int B_BYTES = NBUF * BL_BYTES;
constexpr int NEPI = 8;
constexpr int NISS = 2;
constexpr int THREADS = (NEPI + NISS) * 32;
constexpr uint32_t TMEM_COLS = 256;
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr int kMaxImages = 64;
static_assert(NBLK * 32 <= static_cast<int>(TMEM_COLS), "one 32-column accumulator per block");

// ACNetLegacy: layer 0, eight 3x3 8->8 layers (ReLU), 2x2 transposed conv.
// PART 0: the whole network in one launch.
struct NetLegacy
{
    static constexpr int NL = 9;  // MMA layers (3x3 convolutions)
    static constexpr bool ACN8 = false;
    static constexpr int PART = 0;
};
// The network split in two launches at layer K (fusion depth K + (9 - K)):
// the head runs layers 0 .. K-1 from the image and writes layer K-1's
// 16-bit activations of its tile to an 8-channel map in global memory (the
// values the whole-network kernel keeps in shared memory); the tail reads
// the map, runs layers K .. 8, the transposed conv and the colour merge.
template <int K>
struct NetLegacyHead
{
    static constexpr int NL = K;
    static constexpr bool ACN8 = false;
    static constexpr int PART = 1;
};
template <int K>
struct NetLegacyTail
{
    static constexpr int NL = 9 - K;
    static constexpr bool ACN8 = false;
    static constexpr int PART = 2;
};
// ACNet<8> with B blocks: layer 0, B 3x3 8->8 layers (PReLU), conv3x3 8->4.
template <int B>
struct NetAcn8
{
    static constexpr int NL = B + 2;
    static constexpr bool ACN8 = true;
    static constexpr int PART = 0;
};
// ACNet<8> split at layer K (K <= B, so the head ends on a PReLU layer): the
// head writes layer K-1's activations after PReLU; the tail runs layers
// K .. B and the conv 8->4.
template <int B, int K>
struct NetAcn8Head
{
    static constexpr int NL = K;
    static constexpr bool ACN8 = true;
    static constexpr int PART = 1;
    static_assert(K >= 1 && K <= B, "the head ends on a PReLU layer");
};
template <int B, int K>
struct NetAcn8Tail
{
    static constexpr int NL = B + 2 - K;
    static constexpr bool ACN8 = true;
    static constexpr int PART = 2;
};

// COL: the tile ends in the colour merge (its chroma sums must fit the
// dead activation buffer); a head part's tiles do not.
// XE: extra window columns on each side beyond the halo.  A layer sums an
// output's three horizontal taps in two MMAs, grouped (2 + 1) or (1 + 2) by
// the pixel's column parity in the window, and the FP32 accumulator rounds
// between them; with TW even every tile of a shape puts an image column at
// the same parity, and shapes of one network with the same parity of
// HALO + XE give identical bytes.
template <int TW_, int TH_, int HALO_, bool COL_ = true, int XE_ = 0>
struct Geo
{
    static constexpr int TW = TW_, TH = TH_, HALO = HALO_, XE = XE_;
    static constexpr int HX = HALO + XE;  // window columns left of the tile
    static constexpr int WW = TW + 2 * HX, WH = TH + 2 * HALO;
    static constexpr int QPR = WW / 4;  // quads per window row
    static constexpr int PADQ = QPR + 2;
    static constexpr int PLANE_BYTES = (PADQ + NBLK * 128 + PADQ) * 16;
    static constexpr int ACT_BYTES = 4 * PLANE_BYTES;
    static constexpr int UVW = TW + 4, UVH = TH + 4;
    static constexpr int UVX0 = HX - 2, UVY0 = HALO - 2;  // chroma region origin in the window
    static_assert(WW % 4 == 0, "window rows hold whole quads");
    static_assert(TW % 2 == 0, "each image column at one window column parity");
    static_assert(WW * WH <= NBLK * 512, "window must fit the quad blocks");
    static_assert(!COL_ || UVH * 2 * TW * 3 * 4 <= ACT_BYTES, "chroma sums must fit the activation buffer");
    static_assert(PADQ >= QPR + 1, "taps of the first and last rows stay inside the planes");
    // Bytes per row of the TMA-staged input window of a C-channel u8 image:
    // the window's WW * C bytes plus up to 15 bytes in front of them (the
    // box starts on a 16-byte boundary), rounded up to 16.
    template <int C>
    static constexpr int stage_bx() { return (WW * C + 15 + 15) / 16 * 16; }
};

template <class G, typename T, int C, int PART = 0>
struct Layout
{
    static constexpr int ACT_OFF = 0;
    static constexpr int B_OFF = G::ACT_BYTES;
    static constexpr int UVW = G::UVW, UVH = G::UVH;
    static constexpr int uv_off = B_OFF + B_BYTES;
    static constexpr int uv_bytes =
        (C == 1 || PART == 1) ? 0 : (UVW * UVH * (C - 1) * static_cast<int>(sizeof(T)) + 15) / 16 * 16;
    static constexpr int lut_off = uv_off + uv_bytes;
    static constexpr int lut_bytes = sizeof(T) == 1 ? 1024 : 0;
    // TMA-staged input window (u8 images of 1 or 3 channels: the box of a
    // window row fits one 256-byte TMA box row, and two CTAs still share an
    // SM); 4-channel and 16/32-bit images load the window directly.
    static constexpr bool STAGE = sizeof(T) == 1 && C != 4 && PART != 2;
    static constexpr int BX = STAGE ? G::template stage_bx<C>() : 0;
    static_assert(BX <= 256, "a staged window row must fit one TMA box row");
    static constexpr int stage_off = (lut_off + lut_bytes + 127) / 128 * 128;
    static constexpr int stage_bytes = STAGE ? G::WH * BX : 0;
    static constexpr int misc_off = stage_off + stage_bytes;
    static constexpr int smem = misc_off + 256;
};

struct Image4
{
    Plane in, out;
    Plane map;   // split network: the 8-channel 16-bit activation map (16 bytes per pixel)
    int tiles_x;
    int tile0;
    int staged;  // the input window is TMA-staged through tmap[image] (u8, 1 or 3 channels)
};

struct Params
{
    const uint4* bw;    // NL packed B matrices in global memory (pack_acnet_tc4_weights)
    float k2[32];
    float bias[NLMAX][8];   // per MMA layer, preloaded into the accumulators
    float alpha[NLMAX][8];  // ACNet<8>: PReLU slopes of layers 0 .. NL - 2
    Phase2 ph;
    int nimg;
    int ntiles;
    int* tile_counter;
    int* status;
    Image4 img[kMaxImages];
    // 2-D tensor maps over the input images as rows of bytes (w * channels
    // by h, the image's pitch), box Layout::BX x WH; used where img[i].staged.
    alignas(64) CUtensorMap tmap[kMaxImages];
};
static_assert(sizeof(Params) <= 32764, "kernel parameters must fit the 32 KB parameter space");

// A layer's PReLU slopes as four packed 16-bit pairs (rounded to nearest),
// converted once per layer.
template <bool BF16>
__device__ __forceinline__ void pack_slopes(const float* a, uint32_t (&s2)[4])
{
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        if constexpr (BF16)
        {
            const __nv_bfloat162 s = __floats2bfloat162_rn(a[2 * i], a[2 * i + 1]);
            s2[i] = *reinterpret_cast<const uint32_t*>(&s);
        }
        else
        {
            const __half2 s = __floats2half2_rn(a[2 * i], a[2 * i + 1]);
            s2[i] = *reinterpret_cast<const uint32_t*>(&s);
        }
    }
}

// PReLU on the packed 16-bit pairs: fma(a, min(x, 0), max(x, 0)) per lane
// of each pair (slopes packed by pack_slopes), four instructions per two values.
template <bool BF16>
__device__ __forceinline__ uint4 pack8_prelu(const float* v, const uint32_t (&s2)[4])
{
    uint32_t r[4];
#pragma unroll
    for (int i = 0; i < 4; i++)
    {
        if constexpr (BF16)
        {
            const __nv_bfloat162 x = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
            const __nv_bfloat162 s = *reinterpret_cast<const __nv_bfloat162*>(&s2[i]);
            const __nv_bfloat162 z = __float2bfloat162_rn(0.0f);
            const __nv_bfloat162 y = __hfma2(s, __hmin2(x, z), __hmax2(x, z));
            r[i] = *reinterpret_cast<const uint32_t*>(&y);
        }
        else
        {
            const __half2 x = __floats2half2_rn(v[2 * i], v[2 * i + 1]);
            const __half2 s = *reinterpret_cast<const __half2*>(&s2[i]);
            const __half2 z = __float2half2_rn(0.0f);
            const __half2 y = __hfma2(s, __hmin2(x, z), __hmax2(x, z));
            r[i] = *reinterpret_cast<const uint32_t*>(&y);
        }
    }
    return make_uint4(r[0], r[1], r[2], r[3]);
}

template <bool BF16>
__device__ __forceinline__ uint4 pack8(const float* v)
{
    if constexpr (BF16)
        return make_uint4(tc::pack_relu_bf16x2(v[0], v[1]), tc::pack_relu_bf16x2(v[2], v[3]),
                          tc::pack_relu_bf16x2(v[4], v[5]), tc::pack_relu_bf16x2(v[6], v[7]));
    else
        return make_uint4(tc::pack_relu_f16x2(v[0], v[1]), tc::pack_relu_f16x2(v[2], v[3]), tc::pack_relu_f16x2(v[4], v[5]),
                          tc::pack_relu_f16x2(v[6], v[7]));
}

// Layer-0 input slot of a luma value: channels (y_hi, y_lo, y_hi, 0, ...).
template <bool BF16>
__device__ __forceinline__ uint4 luma_slot(float y)
{
    if constexpr (BF16)
    {
        const float hi = __bfloat162float(__float2bfloat16_rn(y));
        return make_uint4(tc::pack_bf16x2(y, y - hi), tc::pack_bf16x2(y, 0.0f), 0u, 0u);
    }
    else
    {
        const float hi = __half2float(__float2half_rn(y));
        return make_uint4(tc::pack_f16x2(y, y - hi), tc::pack_f16x2(y, 0.0f), 0u, 0u);
    }
}

// Activation slot of window pixel p: plane p mod 4, quad p / 4.
template <class G>
__device__ __forceinline__ uint4* slot(unsigned char* base, int p)
{
    return reinterpret_cast<uint4*>(base + (p & 3) * G::PLANE_BYTES) + G::PADQ + (p >> 2);
}

__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort_flag)
{
    if (tc::mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = tc::global_timer_ns();
    while (!tc::mbar_try_wait_hint(bar, parity, 20000u))
    {
        if (*abort_flag) return false;
        if (tc::global_timer_ns() - t0 > kWaitNs)
        {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}
__device__ __forceinline__ bool wait_count(const uint32_t* cnt, uint32_t target, volatile int* abort_flag)
{
    if (tc::smem_load_acquire(cnt) >= target) return true;
    const uint64_t t0 = tc::global_timer_ns();
    while (tc::smem_load_acquire(cnt) < target)
    {
        if (*abort_flag) return false;
        if (tc::global_timer_ns() - t0 > kWaitNs)
        {
            *abort_flag = 1;
            return false;
        }
    }
    return true;
}

// Quad blocks whose rows hold the valid pixels of layer l (0..8).
template <class G>
struct LayerRange
{
    static constexpr int WW = G::WW, WH = G::WH;
    int ry0, ry1, rx0, rx1, b0, b1;
    __device__ LayerRange(int l, int ix0, int ix1, int iy0, int iy1)
    {
        ry0 = max(l + 1, iy0);
        ry1 = min(WH - 2 - l, iy1);
        rx0 = max(l + 1 + G::XE, ix0);
        rx1 = min(WW - 2 - l - G::XE, ix1);
        b0 = ((ry0 * WW + rx0) >> 2) >> 7;
        b1 = ((ry1 * WW + rx1) >> 2) >> 7;
    }
};

template <class G, class NET, typename T, int C, bool BF16>
__global__ void __launch_bounds__(THREADS, 2) acnet_tc4_kernel(const __grid_constant__ Params P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    using L = Layout<G, T, C, NET::PART>;
    constexpr int NL = NET::NL, LAST = NL - 1, HALO = G::HALO, HX = G::HX;
    static_assert(HALO == NL && NL <= NLMAX, "one halo pixel per 3x3 layer");
    constexpr int TW = G::TW, TH = G::TH, WW = G::WW, WH = G::WH, QPR = G::QPR, PADQ = G::PADQ;
    constexpr int PLANE_BYTES = G::PLANE_BYTES, ACT_BYTES = G::ACT_BYTES;
    constexpr int UVW = G::UVW, UVH = G::UVH, UVX0 = G::UVX0, UVY0 = G::UVY0;
    T* uvs = reinterpret_cast<T*>(smem + L::uv_off);
    float* lut = reinterpret_cast<float*>(smem + L::lut_off);
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + L::misc_off);         // [NBLK]
    uint64_t* round_bar = reinterpret_cast<uint64_t*>(smem + L::misc_off + 64);  // [NROUND]
    uint64_t* bbar = reinterpret_cast<uint64_t*>(smem + L::misc_off + 96);       // [NBUF]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::misc_off + 120);
    volatile int* tile_slot = reinterpret_cast<volatile int*>(smem + L::misc_off + 124);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + L::misc_off + 128);
    uint32_t* gbar = reinterpret_cast<uint32_t*>(smem + L::misc_off + 132);
    uint64_t* tbar = reinterpret_cast<uint64_t*>(smem + L::misc_off + 136);  // staging load of a window
    volatile int* next_slot = reinterpret_cast<volatile int*>(smem + L::misc_off + 144);
    unsigned char* act = smem + L::ACT_OFF;
    unsigned char* bring = smem + L::B_OFF;
    unsigned char* stage = smem + L::stage_off;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool mma_warp = warp >= NEPI;
    const bool loader = warp == NEPI && lane == 0;  // streams the B ring

    // ---- one-time set-up ----
    if (tid == 0)
    {
        for (int b = 0; b < NBLK; b++) tc::mbar_init(&mma_bar[b], 1);
        // two blocks x four lane-quarter warps arrive per round and layer
        for (int r = 0; r < NROUND; r++) tc::mbar_init(&round_bar[r], 8);
        for (int i = 0; i < NBUF; i++) tc::mbar_init(&bbar[i], 1);
        tc::mbar_init(tbar, 1);
        tc::fence_mbar_init();
        *abort_flag = 0;
        *gbar = 0;
    }
    if constexpr (sizeof(T) == 1)
        if (tid < 256) lut[tid] = __fdiv_rn(static_cast<float>(tid), 255.0f);
    // The activation buffer starts at zero (finite values only: see the
    // clearing of the pads in the prologue).
    for (int i = tid; i < ACT_BYTES / 16; i += THREADS) reinterpret_cast<uint4*>(act)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    // the B ring: layers 0 and 1 of the first tile
    uint32_t issued = 0;  // B loads issued by the loader (layer counter of the next one)
    if (loader)
    {
        for (int g = 0; g < 2; g++)
        {
            tc::mbar_arrive_expect_tx(&bbar[g], BL_BYTES);
            tc::bulk_load(bring + g * BL_BYTES, P.bw + g * (BL_BYTES / 16), BL_BYTES, &bbar[g]);
        }
        issued = 2;
    }
    if (warp == 0)
    {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    constexpr uint32_t IDESC = tc::idesc_f16(128, 32, BF16);

    uint32_t layers_done = 0;  // layers completed by this CTA over all its tiles
    uint32_t gbar_gen = 0;
    uint32_t stage_waits = 0;   // staging loads waited on (every thread alike)
    uint32_t stage_issued = 0;  // staging loads issued (thread 0)
    // Thread 0 takes the CTA's next tile from the queue (the first one here,
    // each following one during the last layer of the current tile); when
    // the tile's image is staged it starts the TMA load of the tile's input
    // window (rows gy0 .. gy0 + WH - 1, bytes from the 16-byte boundary at or
    // before column gx0; outside the image the box reads zeros, which the
    // prologue never uses) into the staging buffer, so the load overlaps the
    // current tile's last layer.
    auto take_tile = [&](volatile int* slot) {
        const int t = *abort_flag ? P.ntiles : atomicAdd(P.tile_counter, 1);
        *slot = t;
        if constexpr (L::STAGE)
        {
            if (t < P.ntiles)
            {
                int j = 0;
                while (j + 1 < P.nimg && P.img[j + 1].tile0 <= t) j++;
                const Image4& J = P.img[j];
                if (J.staged)
                {
                    const int loc = t - J.tile0;
                    const int sx = ((loc % J.tiles_x) * TW - HX) * C, sy = (loc / J.tiles_x) * TH - HALO;
                    tc::mbar_arrive_expect_tx(tbar, static_cast<uint32_t>(WH * L::BX));
                    tc::tma_load_2d(stage, &P.tmap[j], sx & ~15, sy, tbar);
                    stage_issued++;
                }
            }
        }
    };
    if (tid == 0) take_tile(tile_slot);
    for (;;)
    {
        __syncthreads();
        const int tile = *tile_slot;
        if (tile >= P.ntiles) break;
        int im = 0;
        while (im + 1 < P.nimg && P.img[im + 1].tile0 <= tile) im++;
        const Image4& I = P.img[im];
        const int local = tile - I.tile0;
        const int gx0 = (local % I.tiles_x) * TW - HX, gy0 = (local / I.tiles_x) * TH - HALO;
        const int W = I.in.w, H = I.in.h;
        const int ix0 = max(0, -gx0), ix1 = min(WW - 1, W - 1 - gx0);
        const int iy0 = max(0, -gy0), iy1 = min(WH - 1, H - 1 - gy0);
        const bool edges = ix0 > 0 || ix1 < WW - 1 || iy0 > 0 || iy1 < WH - 1;
        const bool wide = ((reinterpret_cast<uintptr_t>(I.out.ptr) | static_cast<uintptr_t>(I.out.pitch)) &
                           (store_px2_align<T, C>() - 1)) == 0;

        if constexpr (NET::PART == 2)
        {
            // ---- prologue of a tail part: the window's layer-K input from the
            // 16-bit activation map (clamped: taps that leave the image read
            // the edge pixel, the clamp-to-edge of the intermediate map), and
            // the chroma region from the source image.  ACNetLegacy's tail
            // copies the map pixels straight to their slots by cp.async: all
            // of a thread's copies are in flight at once, no registers held,
            // while the thread computes its part of the chroma region (the
            // 8-frame 1080p RGB step measured 0.5 % faster).  ACNet<8>'s tail
            // keeps register loads, which measured 1-3 % faster there ----
            for (int i = tid; i < WW * WH; i += THREADS)
            {
                const int wy = i / WW, wx = i - wy * WW;
                const int gx = clampi(gx0 + wx, 0, W - 1), gy = clampi(gy0 + wy, 0, H - 1);
                const unsigned char* src = row_ptr<unsigned char>(I.map.ptr, I.map.pitch, gy) + gx * 16;
                if constexpr (NET::ACN8) *slot<G>(act, i) = *reinterpret_cast<const uint4*>(src);
                else tc::cp_async16(slot<G>(act, i), src);
            }
            if constexpr (C > 1)
                for (int e = tid; e < UVW * UVH; e += THREADS)
                {
                    const int uy = e / UVW, ux = e - uy * UVW;
                    const int gx = clampi(gx0 + UVX0 + ux, 0, W - 1), gy = clampi(gy0 + UVY0 + uy, 0, H - 1);
                    const T* sp = row_ptr<T>(I.in.ptr, I.in.pitch, gy) + gx * C;
                    T px[C], yq, uvq[C - 1];
#pragma unroll
                    for (int c = 0; c < C; c++) px[c] = sp[c];
                    rgb_to_yuv_q_lut<T, C>(px, yq, uvq, lut);
#pragma unroll
                    for (int c = 0; c < C - 1; c++) uvs[e * (C - 1) + c] = uvq[c];
                }
            if constexpr (!NET::ACN8) tc::cp_async_wait_all();  // this thread's map copies landed (the barrier below shares them)
        }
        else
        {
        // ---- prologue (all warps): window luma as layer-0 input slots (+ chroma region) ----
        // A staged window is read from shared memory once its TMA load
        // completed (bounded wait); otherwise straight from the image.
        bool staged = false;
        if constexpr (L::STAGE)
        {
            if (I.staged)
            {
                staged = true;
                wait_bar(tbar, stage_waits & 1u, abort_flag);
                stage_waits++;
            }
        }
        const int sx0 = (gx0 * C) & ~15;  // first byte column of the staged box
        constexpr int PER = (WW * WH + THREADS - 1) / THREADS;
        for (int k0 = 0; k0 < PER; k0 += 4)
        {
            T px[4][C];
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                const int i = tid + (k0 + k) * THREADS;
                if (i < WW * WH)
                {
                    const int wy = i / WW, wx = i - wy * WW;
                    const int gx = clampi(gx0 + wx, 0, W - 1), gy = clampi(gy0 + wy, 0, H - 1);
                    const T* src;
                    if constexpr (L::STAGE)
                        src = staged ? reinterpret_cast<const T*>(stage + (gy - gy0) * L::BX + gx * C - sx0)
                                     : row_ptr<T>(I.in.ptr, I.in.pitch, gy) + gx * C;
                    else
                        src = row_ptr<T>(I.in.ptr, I.in.pitch, gy) + gx * C;
#pragma unroll
                    for (int c = 0; c < C; c++) px[k][c] = src[c];
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
            {
                const int i = tid + (k0 + k) * THREADS;
                if (i >= WW * WH) continue;
                T yq;
                if constexpr (C == 1) yq = px[k][0];
                else
                {
                    const int wy = i / WW, wx = i - wy * WW;
                    T uvq[C - 1];
                    rgb_to_yuv_q_lut<T, C>(px[k], yq, uvq, lut);
                    const int ux = wx - UVX0, uy = wy - UVY0;
                    if constexpr (NET::PART == 0)
                        if (ux >= 0 && ux < UVW && uy >= 0 && uy < UVH)
                        {
#pragma unroll
                            for (int c = 0; c < C - 1; c++) uvs[(uy * UVW + ux) * (C - 1) + c] = uvq[c];
                        }
                }
                // clamped loads: taps that leave the image read the edge pixel
                *slot<G>(act, i) = luma_slot<BF16>(to_float_lut<T>(yq, lut));
            }
        }
        }
        // Layer 0's bias into the accumulators of the blocks this warp drains.
        if (!mma_warp)
        {
            float bv[8];
#pragma unroll
            for (int c = 0; c < 8; c++) bv[c] = P.bias[0][c];
#pragma unroll 1
            for (int r = 0; r < NROUND; r++)
                tc::tmem_st32_dup8(tmem + (static_cast<uint32_t>((warp & 3) * 32) << 16) +
                                       static_cast<uint32_t>((2 * r + (warp >> 2)) * 32),
                                   bv);
            tc::tmem_wait_st();
        }
        // The planes' pads and unused tails are read with zero weights by the
        // window's first and last rows; the previous tile's chroma pass may
        // have left non-finite bit patterns there, so they are cleared.
        {
            constexpr int TAIL = PADQ + NBLK * 128 - WW * WH / 4;  // slots after the window in a plane
            constexpr int NZ = PADQ + TAIL;                        // per plane
            for (int i = tid; i < 4 * NZ; i += THREADS)
            {
                const int pl = i / NZ, k = i - pl * NZ;
                reinterpret_cast<uint4*>(act + pl * PLANE_BYTES)[k < PADQ ? k : WW * WH / 4 + k] = make_uint4(0, 0, 0, 0);
            }
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();

        if (mma_warp)
        {
            if (lane == 0)
            {
                // A descriptors of block 0, tap row 0: chunk 0 = (P0[r - QPR],
                // P3[r - QPR - 1]), chunk 1 = (P1[r - QPR], P2[r - QPR]); chunk 2
                // is chunk 0 one slot on.  Block b, tap row dy: + 128 b + QPR dy
                // slots.  B of (slot, dy, chunk c): + (slot BL_BYTES + 1024 (3 dy + c)) / 16.
                const uint32_t act_u = tc::smem_u32(act);
                const uint64_t a0 = tc::smem_desc(act_u + (PADQ - QPR) * 16, 3 * PLANE_BYTES - 16, 128);
                const uint64_t a1 = tc::smem_desc(act_u + PLANE_BYTES + (PADQ - QPR) * 16, PLANE_BYTES, 128);
                const uint64_t bd0 = tc::smem_desc(tc::smem_u32(bring), 512, 128);
                const int blk = warp - NEPI;  // this issuer's block of each round: 2 r + blk
                for (int l = 0; l < NL; l++)
                {
                    const uint32_t gl = layers_done + static_cast<uint32_t>(l);  // layer count over the CTA's tiles
                    const LayerRange<G> R(l, ix0, ix1, iy0, iy1);
                    // this layer's B in the ring
                    bool ok = wait_bar(&bbar[gl % NBUF], (gl / NBUF) & 1u, abort_flag);
                    const uint64_t bd = bd0 + static_cast<uint64_t>(((gl % NBUF) * BL_BYTES) >> 4);
                    const uint32_t rpar = (gl - 1u) & 1u;  // round barriers: layer l-1
                    for (int r = 0; r < NROUND; r++)
                    {
                        bool rok = true;
                        if (l >= 1) rok = wait_bar(&round_bar[min(r + 1, NROUND - 1)], rpar, abort_flag);
                        tc::fence_after_sync();
                        // every MMA of layer gl-1 has completed once layer l's
                        // last round may start (or at a tile's first layer):
                        // its ring slot takes layer gl+2
                        if (loader && (l == 0 ? r == 0 : r == NROUND - 1))
                        {
                            const uint32_t g2 = gl + 2u;
                            if (g2 == issued)
                            {
                                tc::mbar_arrive_expect_tx(&bbar[g2 % NBUF], BL_BYTES);
                                tc::bulk_load(bring + (g2 % NBUF) * BL_BYTES, P.bw + (g2 % NL) * (BL_BYTES / 16), BL_BYTES,
                                              &bbar[g2 % NBUF]);
                                issued++;
                            }
                        }
                        const int b = 2 * r + blk;
                        if (ok && rok && b >= R.b0 && b <= R.b1)
                        {
                            const uint32_t d = tmem + static_cast<uint32_t>(b * 32);
#pragma unroll
                            for (int dy = 0; dy < 3; dy++)
                            {
                                const uint64_t off = static_cast<uint64_t>(b * 128 + dy * QPR);
                                const uint64_t bdy = bd + static_cast<uint64_t>(dy * 3 * (CHUNK_BYTES >> 4));
                                tc::mma_f16(d, a0 + off, bdy, IDESC, 1u);
                                tc::mma_f16(d, a1 + off, bdy + (CHUNK_BYTES >> 4), IDESC, 1u);
                                tc::mma_f16(d, a0 + off + 1, bdy + 2 * (CHUNK_BYTES >> 4), IDESC, 1u);
                            }
                        }
                        tc::mma_commit(&mma_bar[b]);
                    }
                }
            }
            __syncwarp();
        }
        else
        {
            const int q = warp & 3, g = warp >> 2;
            for (int l = 0; l < NL; l++)
            {
                // Near the end of the tile (the prologue read the staging
                // buffer long before): take the next tile and start its
                // window's load, late enough not to hold a tile another CTA
                // could start sooner.
                if (l == LAST && tid == 0) take_tile(next_slot);
                __syncwarp();
                const uint32_t parity = (layers_done + static_cast<uint32_t>(l)) & 1u;
                const LayerRange<G> R(l, ix0, ix1, iy0, iy1);
                uint32_t slopes[4] = {0u, 0u, 0u, 0u};
                if constexpr (NET::ACN8)
                    if (l < LAST || NET::PART == 1) pack_slopes<BF16>(P.alpha[l], slopes);
                float* Hs = reinterpret_cast<float*>(act);  // last layer: the activations are dead once its MMAs completed
                if constexpr (C > 1 && NET::PART != 1)
                {
                    if (l == LAST)
                    {
                        // the horizontal chroma pass once every layer-8 MMA completed
                        bool last = true;
                        for (int i = 0; i < NISS; i++) last = wait_bar(&mma_bar[NBLK - 2 + i], parity, abort_flag) && last;
                        const bool ok = __all_sync(0xffffffffu, last ? 1 : 0);
                        if (ok)
                            for (int e = tid; e < UVH * TW; e += NEPI * 32)
                            {
                                const int r = e / TW, i = e - r * TW;
                                chroma_hpass2<T, C - 1>(uvs + r * UVW * (C - 1), i, P.ph, Hs + (r * 2 * TW + 2 * i) * (C - 1));
                            }
                        // bounded barrier of the epilogue warps
                        __syncwarp();
                        gbar_gen++;
                        if (lane == 0) tc::smem_add_release(gbar, 1);
                        wait_count(gbar, NEPI * gbar_gen, abort_flag);
                        __syncwarp();
                    }
                }
                for (int rr = 0; rr < NROUND; rr++)
                {
                    const int b = 2 * rr + g;
                    // in-place update: blocks b-1 and b+1 read rows that b overwrites
                    bool got = wait_bar(&mma_bar[b], parity, abort_flag);
                    if (b > 0) got = wait_bar(&mma_bar[b - 1], parity, abort_flag) && got;
                    if (b + 1 < NBLK) got = wait_bar(&mma_bar[b + 1], parity, abort_flag) && got;
                    const bool done = __all_sync(0xffffffffu, got ? 1 : 0);
                    tc::fence_after_sync();
                    if (done && b >= R.b0 && b <= R.b1)
                    {
                        const uint32_t ta = tmem + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(b * 32);
                        const int r = b * 128 + q * 32 + lane;  // this lane's quad
                        const int y = (4 * r) / WW, x0 = 4 * r - y * WW;
                        const bool row_ok = y >= R.ry0 && y <= R.ry1;
#pragma unroll
                        for (int half = 0; half < 2; half++)
                        {
                            float v[16];
                            tc::tmem_ld16(ta + static_cast<uint32_t>(16 * half), v);
                            tc::tmem_wait_ld();
                            if (half == 1 && l < LAST)
                            {
                                // both halves read: the next layer's bias into the accumulator
                                float nb[8];
#pragma unroll
                                for (int c = 0; c < 8; c++) nb[c] = P.bias[l + 1][c];
                                tc::tmem_st32_dup8(ta, nb);
                                tc::tmem_wait_st();
                            }
#pragma unroll
                            for (int kk = 0; kk < 2; kk++)
                            {
                                const int k = 2 * half + kk;
                                const int x = x0 + k, p = 4 * r + k;
                                if (!row_ok || x < R.rx0 || x > R.rx1) continue;
                                if (l < LAST)
                                {
                                    uint4 val;
                                    if constexpr (NET::ACN8)
                                        val = pack8_prelu<BF16>(v + 8 * kk, slopes);
                                    else
                                        val = pack8<BF16>(v + 8 * kk);
                                    *slot<G>(act, p) = val;
                                    // clamp-to-edge for the next layer (only tiles at an image edge)
                                    if (!edges) continue;
                                    const bool xl = x == ix0 && x > 0, xr = x == ix1 && x < WW - 1;
                                    const bool yt = y == iy0 && y > 0, yb = y == iy1 && y < WH - 1;
                                    if (xl) *slot<G>(act, p - 1) = val;
                                    if (xr) *slot<G>(act, p + 1) = val;
                                    if (yt)
                                    {
                                        *slot<G>(act, p - WW) = val;
                                        if (xl) *slot<G>(act, p - WW - 1) = val;
                                        if (xr) *slot<G>(act, p - WW + 1) = val;
                                    }
                                    if (yb)
                                    {
                                        *slot<G>(act, p + WW) = val;
                                        if (xl) *slot<G>(act, p + WW - 1) = val;
                                        if (xr) *slot<G>(act, p + WW + 1) = val;
                                    }
                                }
                                else if constexpr (NET::PART == 1)
                                {
                                    // head part: layer K-1's activations of the tile
                                    // (this range is the tile inside the image) to the map
                                    uint4 val;
                                    if constexpr (NET::ACN8)
                                        val = pack8_prelu<BF16>(v + 8 * kk, slopes);
                                    else
                                        val = pack8<BF16>(v + 8 * kk);
                                    *reinterpret_cast<uint4*>(row_ptr_w<unsigned char>(I.map.ptr, I.map.pitch, gy0 + y) +
                                                              (gx0 + x) * 16) = val;
                                }
                                else
                                {
                                    T o[2][2];
                                    if constexpr (NET::ACN8)
                                    {
                                        // conv3x3 8 -> 4 (+ bias, in the accumulator), pixel
                                        // shuffle, + the source pixel's luma (nearest), fromFloat
                                        const int gx = gx0 + x, gy = gy0 + y;
                                        const T* sp = row_ptr<T>(I.in.ptr, I.in.pitch, gy) + gx * C;
                                        T yq;
                                        if constexpr (C == 1) yq = sp[0];
                                        else
                                        {
                                            T px[C], uvq[C - 1];
#pragma unroll
                                            for (int c = 0; c < C; c++) px[c] = sp[c];
                                            rgb_to_yuv_q_lut<T, C>(px, yq, uvq, lut);
                                        }
                                        const float nearv = to_float_lut<T>(yq, lut);
#pragma unroll
                                        for (int n = 0; n < 4; n++)
                                            o[n >> 1][n & 1] = from_float<T>((v[8 * kk + n] + v[8 * kk + n + 4]) + nearv);
                                    }
                                    else
                                    {
                                        float s[8];
#pragma unroll
                                        for (int c = 0; c < 8; c++) s[c] = fmaxf(v[8 * kk + c], 0.0f);
#pragma unroll
                                        for (int dy = 0; dy < 2; dy++)
#pragma unroll
                                            for (int dx = 0; dx < 2; dx++)
                                            {
                                                const int ko = 8 * (dy * 2 + dx);
                                                float d = s[0] * P.k2[ko];
#pragma unroll
                                                for (int c = 1; c < 7; c++) d = fmaf(s[c], P.k2[ko + c], d);
                                                if constexpr (sizeof(T) < 4) o[dy][dx] = from_unit<T>(fma_sat(s[7], P.k2[ko + 7], d));
                                                else o[dy][dx] = from_float<T>(fmaf(s[7], P.k2[ko + 7], d));
                                            }
                                    }
                                    const int ox = 2 * (gx0 + x), oy = 2 * (gy0 + y);
                                    T* row0 = row_ptr_w<T>(I.out.ptr, I.out.pitch, oy) + ox * C;
                                    T* row1 = row_ptr_w<T>(I.out.ptr, I.out.pitch, oy + 1) + ox * C;
                                    if constexpr (C == 1)
                                    {
                                        row0[0] = o[0][0];
                                        row0[1] = o[0][1];
                                        row1[0] = o[1][0];
                                        row1[1] = o[1][1];
                                    }
                                    else merge_block2_hv<T, C>(Hs, 2 * TW, x - HX, y - HALO, P.ph, o, row0, row1, wide, lut);
                                }
                            }
                        }
                    }
                    // publish: activations visible to the tensor core, tensor-memory accesses done
                    tc::fence_proxy_async_smem();
                    tc::fence_before_sync();
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&round_bar[rr]);
                }
            }
        }
        layers_done += NL;
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (tid == 0) *tile_slot = *next_slot;
    }
    // B loads still in flight (issued ahead for tiles that did not come) must
    // land before the CTA exits; bounded by time, not cut short by an abort.
    if (loader)
        for (uint32_t g2 = layers_done; g2 < issued; g2++)
            if (!tc::mbar_wait_ns(&bbar[g2 % NBUF], (g2 / NBUF) & 1u, kWaitNs)) *abort_flag = 1;
    // likewise a staging load whose tile was not processed (after an abort)
    if (tid == 0 && stage_issued > stage_waits && !tc::mbar_wait_ns(tbar, stage_waits & 1u, kWaitNs)) *abort_flag = 1;
    if (tid == 0 && *abort_flag) atomicExch(P.status, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

// Host: the tensor maps of the images whose input windows the kernel stages
// by TMA (u8 with 1 or 3 channels, 16-byte aligned base and pitch; the
// others keep img[i].staged = 0 and are loaded directly).
// AC_GB300_TMA_IN=0 turns staging off (a check that both paths agree).
template <class G>
inline void stage_maps(Params& p, int n, const Plane* in)
{
    for (int i = 0; i < n; i++) p.img[i].staged = 0;
    const int c = in[0].channels;
    if (n <= 0 || in[0].type != kU8 || c == 4) return;
    if (const char* e = std::getenv("AC_GB300_TMA_IN"))
        if (std::atoi(e) == 0) return;
    const int bx = c == 1 ? G::template stage_bx<1>() : G::template stage_bx<3>();
    for (int i = 0; i < n; i++)
        if (encode_tmap_2d(&p.tmap[i], in[i].ptr, 1, in[i].w * c, in[i].h, in[i].pitch, bx, G::WH)) p.img[i].staged = 1;
}

template <class G, class NET, typename T, int C, bool BF16>
cudaError_t launch_typed(const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    // one-time set-up per device, thread-safe
    const LaunchSetup setup = device_once([] {
        cudaError_t err = cudaFuncSetAttribute(acnet_tc4_kernel<G, NET, T, C, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               Layout<G, T, C, NET::PART>::smem);
        if (err != cudaSuccess) return LaunchSetup{err, 0, 0};
        err = cudaFuncSetAttribute(acnet_tc4_kernel<G, NET, T, C, BF16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared);
        if (err != cudaSuccess) return LaunchSetup{err, 0, 0};
        // CTAs per SM from shared memory, registers and threads (as for the
        // pair kernel: two CTAs of 256 tensor-memory columns share an SM).
        cudaFuncAttributes fa;
        err = cudaFuncGetAttributes(&fa, acnet_tc4_kernel<G, NET, T, C, BF16>);
        if (err != cudaSuccess) return LaunchSetup{err, 0, 0};
        int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0;
        if ((err = cudaGetDevice(&dev)) != cudaSuccess) return LaunchSetup{err, 0, 0};
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
        const int regs_cta = (fa.numRegs + 7) / 8 * 8 * THREADS;
        const int need_smem = Layout<G, T, C, NET::PART>::smem + static_cast<int>(fa.sharedSizeBytes) + reserved;
        const int per_sm = (2 * need_smem <= smem_sm && 2 * regs_cta <= regs_sm && 2 * TMEM_COLS <= 512) ? 2 : 1;
        if (std::getenv("AC_GB300_DEBUG"))
            std::fprintf(stderr, "tc4 <%d,%d,%d>: %d CTAs per SM, %d bytes shared, %d registers\n", static_cast<int>(sizeof(T)),
                         C, BF16 ? 1 : 0, per_sm, Layout<G, T, C, NET::PART>::smem, fa.numRegs);
        return LaunchSetup{cudaSuccess, per_sm, 0};
    });
    if (setup.err != cudaSuccess) return setup.err;
    const int per_sm = setup.per_sm;
    const int k = per_sm < per_sm_cap ? per_sm : (per_sm_cap < 1 ? 1 : per_sm_cap);
    acnet_tc4_kernel<G, NET, T, C, BF16><<<grid * k, THREADS, Layout<G, T, C, NET::PART>::smem, stream>>>(p);
    return cudaGetLastError();
}

template <class G, class NET, typename T, bool BF16>
cudaError_t launch_channels(int c, const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    switch (c)
    {
    case 1: return launch_typed<G, NET, T, 1, BF16>(p, grid, per_sm_cap, stream);
    case 3: return launch_typed<G, NET, T, 3, BF16>(p, grid, per_sm_cap, stream);
    case 4: return launch_typed<G, NET, T, 4, BF16>(p, grid, per_sm_cap, stream);
    default: return cudaErrorInvalidValue;
    }
}

template <class G, class NET>
cudaError_t launch_shape(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    switch (type)
    {
    case kU8:
        return bf16 ? launch_channels<G, NET, uint8_t, true>(c, p, grid, per_sm_cap, stream)
                    : launch_channels<G, NET, uint8_t, false>(c, p, grid, per_sm_cap, stream);
    case kU16:
        return bf16 ? launch_channels<G, NET, uint16_t, true>(c, p, grid, per_sm_cap, stream)
                    : launch_channels<G, NET, uint16_t, false>(c, p, grid, per_sm_cap, stream);
    case kF32:
        return bf16 ? launch_channels<G, NET, float, true>(c, p, grid, per_sm_cap, stream)
                    : launch_channels<G, NET, float, false>(c, p, grid, per_sm_cap, stream);
    default: return cudaErrorInvalidValue;
    }
}

using GeoHead = Geo<54, 54, 5, false>;  // ACNetLegacy split at layer 5: head part, 64 x 64 window
// tail part: 56 x 65 window, one extra column each side (the head's and the
// whole network's column parity); its chroma sums fit the buffer
using GeoTail = Geo<46, 57, 4, true, 1>;
constexpr int kSplitK = 5;
extern template cudaError_t launch_shape<GeoHead, NetLegacyHead<kSplitK>>(int, int, bool, const Params&, int, int, cudaStream_t);
extern template cudaError_t launch_shape<GeoTail, NetLegacyTail<kSplitK>>(int, int, bool, const Params&, int, int, cudaStream_t);
using Geo0 = Geo<46, 46, 9>;     // ACNetLegacy: 64 x 64 window (shape 0, the default)
using GeoQ1 = Geo<62, 33, 9>;    // ACNetLegacy shape 1: 80 x 51 window (wide tiles)
using GeoQ2 = Geo<30, 67, 9>;    // ACNetLegacy shape 2: 48 x 85 window (tall tiles)
static_assert(GeoQ1::HX % 2 == Geo0::HX % 2 && GeoQ2::HX % 2 == Geo0::HX % 2 && GeoHead::HX % 2 == Geo0::HX % 2 &&
                  GeoTail::HX % 2 == Geo0::HX % 2,
              "every ACNetLegacy tiling sums the taps of an image column alike");
// Shapes 1 and 2 are instantiated in k_acnet_tc4_shapes.cu (built in parallel).
extern template cudaError_t launch_shape<GeoQ1, NetLegacy>(int, int, bool, const Params&, int, int, cudaStream_t);
extern template cudaError_t launch_shape<GeoQ2, NetLegacy>(int, int, bool, const Params&, int, int, cudaStream_t);
using GeoA8B4 = Geo<52, 48, 6>;  // ACNet<8> B4: 64 x 60 window (chroma sums of a 52 x 52 tile would not fit)
using GeoA8B8 = Geo<44, 44, 10>; // ACNet<8> B8
// ACNet<8> B8 split at layer 5: head 52 x 54 tiles in a 64 x 64 window, tail
// 44 x 60 tiles in a 56 x 70 window, one extra column each side in both (the
// whole-network B8 windows' column parity)
constexpr int kSplitKA8 = 5;
using GeoA8B8Head = Geo<52, 54, 5, false, 1>;
using GeoA8B8Tail = Geo<44, 60, 5, true, 1>;
static_assert(GeoA8B8Head::HX % 2 == GeoA8B8::HX % 2 && GeoA8B8Tail::HX % 2 == GeoA8B8::HX % 2,
              "every ACNet<8> B8 tiling sums the taps of an image column alike");

// One layer of 3x3 8->8 weights k[n * 72 + tap * 8 + c] (reference NHWC
// order) as the nine N32 x K16 B chunks of the quad GEMM.  Chunk 3 dy + j
// multiplies tap row dy; its K halves hold the 8 channels of the input
// pixels at offsets (0, -1), (+1, +2), (+4, +3) from the row's first pixel
// 4r for j = 0, 1, 2.  Output column n is pixel 4r + n / 8, channel n % 8;
// input offset o feeds output pixel k through tap dx = o - k + 1 (zero
// weight outside 0..2).  Bytes of element (n, kk) in a chunk: (kk / 8) 512 +
// (n / 8) 128 + (n % 8) 16 + (kk % 8) 2 (K-major, no swizzle, leading byte
// offset 512, stride byte offset 128).
void pack_quad_conv8(const float* k, bool bf16, uint16_t* out);
// Layer 0 (1 -> 8, k[n * 9 + tap]) as an 8-channel layer over the input slots
// (y_hi, y_lo, y_hi) with weights (w_hi, w_hi, w_lo).
void pack_quad_layer0(const float* k, bool bf16, uint16_t* out);

}  // namespace tcv4
}  // namespace acgb
