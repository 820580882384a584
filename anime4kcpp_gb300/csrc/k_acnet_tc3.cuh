#pragma once
// Persistent, warp-specialised tensor-core ACNetLegacy x2 kernel over a tile
// queue of one or many images (template over the tile geometry; the shapes
// are instantiated in k_acnet_tc3.cu and k_acnet_tc3_shapes.cu).
//
// Network and clamp semantics: the reference's layer math
// (core/internal/AC/Core/Internal/Processor/CPU/Common.hpp:116-197,344-393),
// every 3x3 layer reading its input map clamped to the image edge.  GEMM
// formulation (pair-interleaved): one GEMM row = two horizontally adjacent
// pixels, N = 2 x 8 output channels = 16, K = 3 tap rows x 4 pixels x 8
// channels.  Activations live as two planes (even / odd pixels), 16 bytes (8
// FP16/BF16 channels) per pixel; a K-major shared-memory descriptor whose
// leading byte offset is the distance between the planes reads a shifted
// view of the window for every tap row, so no im2col copy is made: six
// M128 x N16 x K16 MMAs per 128 pairs and layer, FP32 accumulators in tensor
// memory.  The fused colour prologue / epilogue is that of colour.cuh.  The
// schedule:
//
//  * Two CTAs per SM (one activation buffer and 256 tensor-memory columns
//    each) loop over tiles taken from a global atomic counter; the tiles of
//    every image of a batch form one queue (images of different sizes in one
//    launch).  The packed weights are copied to shared memory once per CTA
//    and the tensor memory is allocated once.  Two CTAs give the SM two MMA
//    issuing threads and two tiles in flight, so one tile's prologue or
//    epilogue overlaps the other's MMAs.
//  * Warps 8 and 9 issue the MMAs (one issuing thread reaches only about
//    half the tensor core's rate for these small MMAs; two saturate it), a
//    round of four pair blocks (4 x 128 GEMM rows) at a time, two blocks
//    each: for layer l and round r both wait on one mbarrier saying the
//    epilogues of layer l-1 have finished round r+1 (and with it every block
//    up to 4r+7; the taps and edge replicas of round r reach blocks 4r-1 ..
//    4r+4), then issue six MMAs per block, block after block (an
//    accumulator's MMAs back to back issue fastest), with descriptors
//    precomputed up to one add, and commit each block to its mbarrier.
//  * Warps 0..7 are the epilogue: two groups of four warps (one warp per
//    tensor-memory lane quarter); group g drains blocks 4r+g and 4r+g+2 of
//    every round as soon as their MMAs completed, adds the bias in FP32 and
//    writes the next layer's activations in place.  In-place is safe because
//    a block's epilogue also waits until the MMAs of the blocks before and
//    after it have completed (they read the rows it overwrites; they may come
//    from the other issuer), and a block's accumulator
//    is overwritten by the next layer only after the round barrier above.
//  * Layer 0 (3x3, 1 -> 8) runs on the tensor core too, as a ninth layer of
//    the same shape: the prologue stores each window pixel's luma in the
//    activation slot as three 16-bit channels (y_hi, y_lo, y_hi, where y_lo =
//    y - y_hi) and the layer's B matrix holds (w_hi, w_hi, w_lo) for them, so
//    the FP32 accumulation of y_hi w_hi + y_lo w_hi + y_hi w_lo carries the
//    layer at close to FP32 accuracy (the dropped y_lo w_lo term is ~2^-22
//    relative for FP16 operands).
//  * The bias rides in the accumulator: before a layer's MMAs the block's
//    tensor-memory columns hold that layer's bias (written with tcgen05.st
//    by the epilogue warp that drained the previous layer's accumulator, or
//    by the prologue for layer 0), and every MMA accumulates onto it.
//  * Every wait is bounded by %globaltimer; a timeout raises a CTA-wide abort
//    flag and the status word, all roles fall through their loops without
//    touching tensor memory, and the CTA frees its tensor memory and exits.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>

#include "colour.cuh"
#include "device_common.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"

namespace acgb {
namespace tcv3 {

constexpr int HALO = 9;
constexpr int NBLK = 16;  // 16 x 128 pairs per window
constexpr int NROUND = NBLK / 4;
constexpr int BL_BYTES = 12 * 256;       // one layer's packed B (pack_pair_conv8)
constexpr int NL = 9;                    // MMA layers: layer 0 and the eight 3x3 8->8 layers
constexpr int LAST = NL - 1;             // the layer followed by the deconvolution
constexpr int B_BYTES = NL * BL_BYTES;
constexpr int NEPI = 8;                   // epilogue warps: two groups of four
constexpr int NISS = 2;                   // MMA issuing warps
constexpr int THREADS = (NEPI + NISS) * 32;
constexpr uint32_t TMEM_COLS = 256;
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr int kMaxImages = 64;
static_assert(NBLK * 16 <= static_cast<int>(TMEM_COLS), "one 16-column accumulator per block");

// Tile geometry: a TW x TH output tile in a (TW + 18) x (TH + 18) window of
// at most NBLK x 128 pixel pairs.
template <int TW_, int TH_>
struct Geo
{
    static constexpr int TW = TW_, TH = TH_;
    static constexpr int WW = TW + 2 * HALO, WH = TH + 2 * HALO;
    static constexpr int PPR = WW / 2;  // pairs per window row
    static constexpr int PADP = PPR + 2 > 40 ? PPR + 2 : 40;
    static constexpr int PLANE_BYTES = (PADP + NBLK * 128 + PADP) * 16;
    static constexpr int ACT_BYTES = 2 * PLANE_BYTES;  // the activation buffer: E plane + O plane
    static constexpr int UVW = TW + 4, UVH = TH + 4;
    static constexpr int UVX0 = HALO - 2;
    static_assert(WW % 2 == 0, "window rows hold whole pairs");
    static_assert(WW * WH / 2 <= NBLK * 128, "window must fit the pair blocks");
    static_assert(UVH * 2 * TW * 3 * 4 <= ACT_BYTES, "chroma sums must fit the activation buffer");
    static_assert(PADP >= PPR + 1, "row above block 0 must stay inside the plane");
};

template <class G, typename T, int C>
struct Layout
{
    static constexpr int ACT_OFF = 0;
    static constexpr int B_OFF = G::ACT_BYTES;
    static constexpr int WW = G::WW, WH = G::WH, UVW = G::UVW, UVH = G::UVH;
    static constexpr int uv_off = B_OFF + B_BYTES;
    static constexpr int uv_bytes = C == 1 ? 0 : (UVW * UVH * (C - 1) * static_cast<int>(sizeof(T)) + 15) / 16 * 16;
    static constexpr int lut_off = uv_off + uv_bytes;
    static constexpr int lut_bytes = sizeof(T) == 1 ? 1024 : 0;
    static constexpr int misc_off = lut_off + lut_bytes;
    static constexpr int smem = misc_off + 256;
};

struct Image3
{
    Plane in, out;
    int tiles_x;
    int tile0;  // index of the image's first tile in the queue
};

struct Params
{
    const uint4* bw;    // NL packed B matrices (pack_acnet_tc3_weights)
    float k2[32];
    float bias[NL][8];  // layers 0..8, preloaded into the accumulators
    Phase2 ph;
    int nimg;
    int ntiles;
    int* tile_counter;
    int* status;
    Image3 img[kMaxImages];
};

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

// Layer-0 input slot of a luma value: channels (y_hi, y_lo, y_hi, 0, ...),
// y_hi = y rounded to the operand type and y_lo = y - y_hi rounded again.
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

// Activation slot of window pixel p in the buffer at `base`.
template <class G>
__device__ __forceinline__ uint4* slot(unsigned char* base, int p)
{
    return reinterpret_cast<uint4*>(base + ((p & 1) ? G::PLANE_BYTES : 0)) + G::PADP + (p >> 1);
}

// Bounded waits that give up at once when the CTA aborted.
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort_flag)
{
    if (tc::mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = tc::global_timer_ns();
    // waiting warps sleep in the barrier unit rather than taking issue slots
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

// Pair blocks whose rows hold the valid pixels of layer l (1..8).
template <class G>
struct LayerRange
{
    static constexpr int WW = G::WW, WH = G::WH;
    int ry0, ry1, rx0, rx1, b0, b1;
    __device__ LayerRange(int l, int ix0, int ix1, int iy0, int iy1)
    {
        ry0 = max(l + 1, iy0);
        ry1 = min(WH - 2 - l, iy1);
        rx0 = max(l + 1, ix0);
        rx1 = min(WW - 2 - l, ix1);
        b0 = ((ry0 * WW + rx0) >> 1) >> 7;
        b1 = ((ry1 * WW + rx1) >> 1) >> 7;
    }
};

template <class G, typename T, int C, bool BF16>
__global__ void __launch_bounds__(THREADS, 2) acnet_tc3_kernel(const __grid_constant__ Params P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    using L = Layout<G, T, C>;
    constexpr int TW = G::TW, TH = G::TH, WW = G::WW, WH = G::WH, PPR = G::PPR, PADP = G::PADP;
    constexpr int PLANE_BYTES = G::PLANE_BYTES, ACT_BYTES = G::ACT_BYTES;
    constexpr int UVW = G::UVW, UVH = G::UVH, UVX0 = G::UVX0;
    constexpr int ACT_OFF = L::ACT_OFF, B_OFF = L::B_OFF;
    T* uvs = reinterpret_cast<T*>(smem + L::uv_off);
    float* lut = reinterpret_cast<float*>(smem + L::lut_off);
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + L::misc_off);         // [NBLK]
    uint64_t* round_bar = reinterpret_cast<uint64_t*>(smem + L::misc_off + 128);  // [NROUND]
    uint64_t* wbar = reinterpret_cast<uint64_t*>(smem + L::misc_off + 192);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::misc_off + 200);
    volatile int* tile_slot = reinterpret_cast<volatile int*>(smem + L::misc_off + 204);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + L::misc_off + 208);
    uint32_t* gbar = reinterpret_cast<uint32_t*>(smem + L::misc_off + 212);
    unsigned char* act = smem + ACT_OFF;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool mma_warp = warp >= NEPI;

    // ---- one-time set-up ----
    if (tid == 0)
    {
        for (int b = 0; b < NBLK; b++) tc::mbar_init(&mma_bar[b], 1);
        // four blocks x four lane-quarter warps arrive per round and layer
        for (int r = 0; r < NROUND; r++) tc::mbar_init(&round_bar[r], 16);
        tc::mbar_init(wbar, 1);
        tc::fence_mbar_init();
        *abort_flag = 0;
        *gbar = 0;
    }
    if constexpr (sizeof(T) == 1)
        if (tid < 256) lut[tid] = __fdiv_rn(static_cast<float>(tid), 255.0f);
    // The activation buffer starts at zero.  Each MMA also reads the
    // neighbouring pair slot of an edge pixel with a zero weight, and a
    // left-over non-finite bit pattern there would turn 0 x Inf into NaN;
    // every value the epilogue writes later is finite.
    for (int i = tid; i < ACT_BYTES / 16; i += THREADS) reinterpret_cast<uint4*>(act)[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    if (tid == 0)
    {
        tc::mbar_arrive_expect_tx(wbar, B_BYTES);
        tc::bulk_load(smem + B_OFF, P.bw, B_BYTES, wbar);
    }
    if (warp == 0)
    {
        tc::tmem_alloc(tmem_slot, TMEM_COLS);
        tc::tmem_relinquish();
    }
    const bool wok = __syncthreads_and(tc::mbar_wait_ns(wbar, 0, kWaitNs) ? 1 : 0) != 0;
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;
    if (!wok && tid == 0) *abort_flag = 1;
    constexpr uint32_t IDESC = tc::idesc_f16(128, 16, BF16);

    uint32_t layers_done = 0;  // layers completed by this CTA over all its tiles
    uint32_t gbar_gen = 0;
    for (;;)
    {
        if (tid == 0) *tile_slot = *abort_flag ? P.ntiles : atomicAdd(P.tile_counter, 1);
        __syncthreads();
        const int tile = *tile_slot;
        if (tile >= P.ntiles) break;
        int im = 0;
        while (im + 1 < P.nimg && P.img[im + 1].tile0 <= tile) im++;
        const Image3& I = P.img[im];
        const int local = tile - I.tile0;
        const int gx0 = (local % I.tiles_x) * TW - HALO, gy0 = (local / I.tiles_x) * TH - HALO;
        const int W = I.in.w, H = I.in.h;
        const int ix0 = max(0, -gx0), ix1 = min(WW - 1, W - 1 - gx0);
        const int iy0 = max(0, -gy0), iy1 = min(WH - 1, H - 1 - gy0);
        const bool edges = ix0 > 0 || ix1 < WW - 1 || iy0 > 0 || iy1 < WH - 1;  // an image edge inside the window
        // output rows aligned for the colour epilogue's wide stores
        const bool wide = ((reinterpret_cast<uintptr_t>(I.out.ptr) | static_cast<uintptr_t>(I.out.pitch)) &
                           (store_px2_align<T, C>() - 1)) == 0;

        // ---- prologue (all warps): window luma as layer-0 input slots (+ chroma region) ----
        // Loads are issued in batches of four pixels per thread before any
        // of them is converted, so their latencies overlap.
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
                    const T* src = row_ptr<T>(I.in.ptr, I.in.pitch, gy) + gx * C;
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
                    const int ux = wx - UVX0, uy = wy - UVX0;
                    if (ux >= 0 && ux < UVW && uy >= 0 && uy < UVH)
                    {
#pragma unroll
                        for (int c = 0; c < C - 1; c++) uvs[(uy * UVW + ux) * (C - 1) + c] = uvq[c];
                    }
                }
                // the window is loaded with clamped coordinates, so taps
                // that leave the image read the edge pixel (clamp-to-edge)
                *slot<G>(act, i) = luma_slot<BF16>(to_float_lut<T>(yq, lut));
            }
        }
        // Layer 0's bias into the accumulators of the blocks this warp drains.
        if (!mma_warp)
        {
            float bv[8];
#pragma unroll
            for (int c = 0; c < 8; c++) bv[c] = P.bias[0][c];
#pragma unroll 1
            for (int k = 0; k < NBLK / 2; k++)
                tc::tmem_st16_dup8(tmem + (static_cast<uint32_t>((warp & 3) * 32) << 16) +
                                       static_cast<uint32_t>((4 * (k >> 1) + (warp >> 2) + 2 * (k & 1)) * 16),
                                   bv);
            tc::tmem_wait_st();
        }
        // The slots around the window (the planes' pads and the unused tail)
        // are read with zero weights by the window's first and last rows;
        // the previous tile's chroma pass may have left non-finite bit
        // patterns there, so they are cleared.
        {
            constexpr int TAIL = G::PADP + NBLK * 128 - WW * WH / 2;  // slots after the window in a plane
            constexpr int NZ = G::PADP + TAIL;                        // per plane
            for (int i = tid; i < 2 * NZ; i += THREADS)
            {
                const int pl = i / NZ, k = i - pl * NZ;
                reinterpret_cast<uint4*>(act + pl * PLANE_BYTES)[k < G::PADP ? k : WW * WH / 2 + k] = make_uint4(0, 0, 0, 0);
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
                // descriptors: A for (block b, tap row dy, half h) = a_desc0 +
                // 128 b + PPR dy + h; B for (layer l, dy, h) = b_desc0 +
                // (BL_BYTES l + 512 (2 dy + h)) / 16
                const uint64_t a_desc0 = tc::smem_desc(tc::smem_u32(act) + (PADP - PPR) * 16, PLANE_BYTES - 16, 128);
                const uint64_t b_desc0 = tc::smem_desc(tc::smem_u32(smem + B_OFF), 256, 128);
                for (int l = 0; l < NL; l++)
                {
                    const LayerRange<G> R(l, ix0, ix1, iy0, iy1);
                    const uint64_t b_desc = b_desc0 + static_cast<uint64_t>((l * BL_BYTES) >> 4);
                    // round barriers: phase of layer l-1 of this tile
                    const uint32_t rpar = (layers_done + static_cast<uint32_t>(l) - 1u) & 1u;
                    for (int r = 0; r < NROUND; r++)
                    {
                        bool ok = true;
                        if (l >= 1) ok = wait_bar(&round_bar[min(r + 1, NROUND - 1)], rpar, abort_flag);
                        tc::fence_after_sync();
                        const int mine = 4 * r + 2 * (warp - NEPI);  // this issuer's two blocks
                        const int lo = max(mine, R.b0), hi = min(mine + 1, R.b1);
                        if (ok)
                            for (int b = lo; b <= hi; b++)
                            {
                                const uint64_t a_desc = a_desc0 + static_cast<uint64_t>(b * 128);
                                const uint32_t d = tmem + static_cast<uint32_t>(b * 16);
#pragma unroll
                                for (int dy = 0; dy < 3; dy++)
#pragma unroll
                                    for (int h = 0; h < 2; h++)
                                        tc::mma_f16(d, a_desc + static_cast<uint64_t>(dy * PPR + h),
                                                    b_desc + static_cast<uint64_t>((2 * dy + h) * 32), IDESC, 1u);
                            }
                        tc::mma_commit(&mma_bar[mine]);
                        tc::mma_commit(&mma_bar[mine + 1]);
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
                const uint32_t parity = (layers_done + static_cast<uint32_t>(l)) & 1u;
                const LayerRange<G> R(l, ix0, ix1, iy0, iy1);
                float* Hs = reinterpret_cast<float*>(act);  // last layer: the activations are dead once its MMAs completed
                if constexpr (C > 1)
                {
                    if (l == LAST)
                    {
                        // the horizontal chroma pass once every layer-8 MMA completed
                        // (the last commit of each issuer)
                        bool last = true;
                        for (int i = 0; i < NISS; i++) last = wait_bar(&mma_bar[NBLK - 3 + 2 * i], parity, abort_flag) && last;
                        const bool ok = __all_sync(0xffffffffu, last ? 1 : 0);
                        if (ok)
                            for (int e = tid; e < UVH * TW; e += NEPI * 32)
                            {
                                // both phases of source column i of region row r
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
#pragma unroll
                    for (int k2 = 0; k2 < 2; k2++)
                    {
                        const int b = 4 * rr + g + 2 * k2;
                        // in-place update: blocks b-1 and b+1 read rows that b overwrites
                        bool got = wait_bar(&mma_bar[b], parity, abort_flag);
                        if (b > 0) got = wait_bar(&mma_bar[b - 1], parity, abort_flag) && got;
                        if (b + 1 < NBLK) got = wait_bar(&mma_bar[b + 1], parity, abort_flag) && got;
                        const bool done = __all_sync(0xffffffffu, got ? 1 : 0);
                        tc::fence_after_sync();
                        if (done && b >= R.b0 && b <= R.b1)
                        {
                            float v[16];
                            const uint32_t ta = tmem + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(b * 16);
                            tc::tmem_ld16(ta, v);
                            tc::tmem_wait_ld();
                            if (l < LAST)
                            {
                                // the next layer's bias into the drained accumulator
                                float nb[8];
#pragma unroll
                                for (int c = 0; c < 8; c++) nb[c] = P.bias[l + 1][c];
                                tc::tmem_st16_dup8(ta, nb);
                                tc::tmem_wait_st();
                            }
                            const int r = b * 128 + q * 32 + lane;
#pragma unroll
                            for (int k = 0; k < 2; k++)
                            {
                                const int p = 2 * r + k;
                                const int y = p / WW, x = p - y * WW;
                                if (y < R.ry0 || y > R.ry1 || x < R.rx0 || x > R.rx1) continue;
                                if (l < LAST)
                                {
                                    const uint4 val = pack8<BF16>(v + 8 * k);
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
                                else
                                {
                                    float s[8];
#pragma unroll
                                    for (int c = 0; c < 8; c++) s[c] = fmaxf(v[8 * k + c], 0.0f);
                                    T o[2][2];
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
                                    else merge_block2_hv<T, C>(Hs, 2 * TW, x - HALO, y - HALO, P.ph, o, row0, row1, wide, lut);
                                }
                            }
                        }
                        // publish: activations visible to the tensor core, tensor-memory reads done
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
    }
    if (tid == 0 && *abort_flag) atomicExch(P.status, 1);
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

template <class G, typename T, int C, bool BF16>
cudaError_t launch_typed(const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    // one-time set-up per device, thread-safe
    const LaunchSetup setup = device_once([] {
        cudaError_t err = cudaFuncSetAttribute(acnet_tc3_kernel<G, T, C, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               Layout<G, T, C>::smem);
        if (err != cudaSuccess) return LaunchSetup{err, 0, 0};
        err = cudaFuncSetAttribute(acnet_tc3_kernel<G, T, C, BF16>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                   cudaSharedmemCarveoutMaxShared);
        if (err != cudaSuccess) return LaunchSetup{err, 0, 0};
        // CTAs per SM from shared memory, registers and threads.  (The
        // occupancy calculator reports one CTA per SM for any kernel that
        // allocates tensor memory; two CTAs of 256 columns each do run
        // side by side.)
        cudaFuncAttributes fa;
        err = cudaFuncGetAttributes(&fa, acnet_tc3_kernel<G, T, C, BF16>);
        if (err != cudaSuccess) return LaunchSetup{err, 0, 0};
        int dev = 0, smem_sm = 0, reserved = 0, regs_sm = 0;
        if ((err = cudaGetDevice(&dev)) != cudaSuccess) return LaunchSetup{err, 0, 0};
        cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev);
        cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
        const int regs_cta = (fa.numRegs + 7) / 8 * 8 * THREADS;
        const int need_smem = Layout<G, T, C>::smem + static_cast<int>(fa.sharedSizeBytes) + reserved;
        const int per_sm = (2 * need_smem <= smem_sm && 2 * regs_cta <= regs_sm && 2 * TMEM_COLS <= 512) ? 2 : 1;
        if (std::getenv("AC_GB300_DEBUG"))
            std::fprintf(stderr, "tc3 <%d,%d,%d>: %d CTAs per SM, %d bytes shared, %d registers\n", static_cast<int>(sizeof(T)),
                         C, BF16 ? 1 : 0, per_sm, Layout<G, T, C>::smem, fa.numRegs);
        return LaunchSetup{cudaSuccess, per_sm, 0};
    });
    if (setup.err != cudaSuccess) return setup.err;
    const int per_sm = setup.per_sm;
    const int k = per_sm < per_sm_cap ? per_sm : (per_sm_cap < 1 ? 1 : per_sm_cap);
    acnet_tc3_kernel<G, T, C, BF16><<<grid * k, THREADS, Layout<G, T, C>::smem, stream>>>(p);
    return cudaGetLastError();
}

template <class G, typename T, bool BF16>
cudaError_t launch_channels(int c, const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    switch (c)
    {
    case 1: return launch_typed<G, T, 1, BF16>(p, grid, per_sm_cap, stream);
    case 3: return launch_typed<G, T, 3, BF16>(p, grid, per_sm_cap, stream);
    case 4: return launch_typed<G, T, 4, BF16>(p, grid, per_sm_cap, stream);
    default: return cudaErrorInvalidValue;
    }
}

// Every element type, channel count and form of one tile geometry.
template <class G>
cudaError_t launch_shape(int type, int c, bool bf16, const Params& p, int grid, int per_sm_cap, cudaStream_t stream)
{
    switch (type)
    {
    case kU8:
        return bf16 ? launch_channels<G, uint8_t, true>(c, p, grid, per_sm_cap, stream)
                    : launch_channels<G, uint8_t, false>(c, p, grid, per_sm_cap, stream);
    case kU16:
        return bf16 ? launch_channels<G, uint16_t, true>(c, p, grid, per_sm_cap, stream)
                    : launch_channels<G, uint16_t, false>(c, p, grid, per_sm_cap, stream);
    case kF32:
        return bf16 ? launch_channels<G, float, true>(c, p, grid, per_sm_cap, stream)
                    : launch_channels<G, float, false>(c, p, grid, per_sm_cap, stream);
    default: return cudaErrorInvalidValue;
    }
}

// The instantiated tile shapes (index = the `shape` argument of the launcher).
using Geo0 = Geo<48, 44>;  // 66 x 62 window, the default
using Geo1 = Geo<64, 31>;  // 82 x 49, wide
using Geo2 = Geo<32, 63>;  // 50 x 81, tall
extern template cudaError_t launch_shape<Geo1>(int, int, bool, const Params&, int, int, cudaStream_t);
extern template cudaError_t launch_shape<Geo2>(int, int, bool, const Params&, int, int, cudaStream_t);

}  // namespace tcv3
}  // namespace acgb
