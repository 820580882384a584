// Persistent, warp-specialised tensor-core ACNetLegacy x2 kernel over a tile
// queue of one or many images.
//
// Network, clamp semantics and the pair-interleaved GEMM formulation are
// those of k_acnet_tc2.cu (reference layer math:
// core/internal/AC/Core/Internal/Processor/CPU/Common.hpp:116-197,344-393);
// the fused colour prologue/epilogue that of colour.cuh.  What changes is the
// schedule:
//
//  * One CTA per SM loops over tiles taken from a global atomic counter; the
//    tiles of every image of a batch form one queue (images of different
//    sizes in one launch).  The packed weights are copied to shared memory
//    once per CTA (bulk copy) and the 512 tensor-memory columns are allocated
//    once.
//  * Accumulators are double-buffered by layer parity in tensor memory
//    (2 x 16 blocks x 16 columns) and activations by layer parity in shared
//    memory (two E/O plane pairs), so layer l+1 can start on block b while
//    layer l is still being drained elsewhere in the window.
//  * Warp 16 issues the MMAs.  For layer l and pair block b it waits until
//    the epilogues of layer l-1 have finished blocks b-2 .. b+2 (the rows the
//    3x3 taps and the edge replicas touch), issues the block's seven MMAs and
//    commits them to that block's mbarrier.  Warps 0..15 are the epilogue:
//    four groups of four warps (one warp per tensor-memory lane quarter),
//    group g drains blocks g, g+4, g+8, g+12 of every layer, each as soon as
//    its MMAs completed, and publishes completion through per-block counters
//    (release/acquire).  The tensor core and the CUDA cores thus work on
//    different blocks at the same time instead of alternating.
//  * Every wait is bounded by %globaltimer; a timeout raises a CTA-wide abort
//    flag and the status word, all roles fall through their loops without
//    touching tensor memory, and the CTA frees its tensor memory and exits.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>

#include "colour.cuh"
#include "device_common.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"

namespace acgb {
namespace tcv3 {

constexpr int TW = 48, TH = 44, HALO = 9;
constexpr int WW = TW + 2 * HALO, WH = TH + 2 * HALO;  // 66 x 62 window
constexpr int PPR = WW / 2;                             // pairs per window row
constexpr int NBLK = 16;                                // 16 x 128 pairs >= 2046
constexpr int PADP = 40;
constexpr int PLANE_BYTES = (PADP + NBLK * 128 + PADP) * 16;
constexpr int ACT_BYTES = 2 * PLANE_BYTES;  // one activation buffer: E plane + O plane
constexpr int BL_BYTES = 14 * 256;
constexpr int NL = 8;
constexpr int B_BYTES = NL * BL_BYTES;
constexpr int NEPI = 16;                 // epilogue warps
constexpr int THREADS = (NEPI + 1) * 32;  // + the MMA warp
constexpr uint32_t TMEM_COLS = 512;
constexpr int UVW = TW + 4, UVH = TH + 4;
constexpr int UVX0 = HALO - 2;
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr int kMaxImages = 64;
static_assert(WW * WH / 2 <= NBLK * 128, "window must fit the pair blocks");
static_assert(UVH * 2 * TW * 3 * 4 <= ACT_BYTES, "chroma sums must fit one activation buffer");

constexpr int ACT0_OFF = 0;
constexpr int ACT1_OFF = ACT_BYTES;
constexpr int B_OFF = 2 * ACT_BYTES;
constexpr int ONES_OFF = B_OFF + B_BYTES;
constexpr int ONES_BYTES = 129 * 16 + 112;
constexpr int RAW_OFF = ONES_OFF + ONES_BYTES;

template <typename T, int C>
struct Layout
{
    static constexpr int raw_bytes = (WW * WH * static_cast<int>(sizeof(T)) + 15) / 16 * 16;
    static constexpr int uv_off = RAW_OFF + raw_bytes;
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
    const uint4* bw;
    float k0[72];
    float b0[8];
    float k2[32];
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

// Activation slot of window pixel p in the buffer at `base`.
__device__ __forceinline__ uint4* slot(unsigned char* base, int p)
{
    return reinterpret_cast<uint4*>(base + ((p & 1) ? PLANE_BYTES : 0)) + PADP + (p >> 1);
}

// Bounded waits that give up at once when the CTA aborted.
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort_flag)
{
    if (tc::mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = tc::global_timer_ns();
    while (!tc::mbar_try_wait(bar, parity))
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

template <typename T, int C, bool BF16>
__global__ void __launch_bounds__(THREADS, 1) acnet_tc3_kernel(const __grid_constant__ Params P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    using L = Layout<T, C>;
    T* raw = reinterpret_cast<T*>(smem + RAW_OFF);
    T* uvs = reinterpret_cast<T*>(smem + L::uv_off);
    float* lut = reinterpret_cast<float*>(smem + L::lut_off);
    uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + L::misc_off);     // [NBLK]
    uint32_t* epi_cnt = reinterpret_cast<uint32_t*>(smem + L::misc_off + 128);  // [NBLK]
    uint64_t* wbar = reinterpret_cast<uint64_t*>(smem + L::misc_off + 192);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::misc_off + 200);
    volatile int* tile_slot = reinterpret_cast<volatile int*>(smem + L::misc_off + 204);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + L::misc_off + 208);
    uint32_t* gbar = reinterpret_cast<uint32_t*>(smem + L::misc_off + 212);
    unsigned char* act0 = smem + ACT0_OFF;
    unsigned char* act1 = smem + ACT1_OFF;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const bool mma_warp = warp == NEPI;

    // ---- one-time set-up ----
    if (tid == 0)
    {
        for (int b = 0; b < NBLK; b++) tc::mbar_init(&mma_bar[b], 1);
        tc::mbar_init(wbar, 1);
        tc::fence_mbar_init();
        for (int b = 0; b < NBLK; b++) epi_cnt[b] = 0;
        *abort_flag = 0;
        *gbar = 0;
    }
    if constexpr (sizeof(T) == 1)
        if (tid < 256) lut[tid] = __fdiv_rn(static_cast<float>(tid), 255.0f);
    if (tid < 129)
    {
        const uint32_t one = BF16 ? 0x3F80u : 0x3C00u;
        reinterpret_cast<uint4*>(smem + ONES_OFF)[tid] = make_uint4(one | (one << 16), 0, 0, 0);
    }
    // Both activation buffers start at zero.  Each MMA also reads the
    // neighbouring pair slot of an edge pixel with a zero weight, and a
    // left-over non-finite bit pattern there would turn 0 x Inf into NaN;
    // every value the epilogue writes later is finite.
    for (int i = tid; i < 2 * ACT_BYTES / 16; i += THREADS) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0, 0, 0, 0);
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
    const uint32_t act0_a = tc::smem_u32(act0), act1_a = tc::smem_u32(act1);
    const uint32_t ones_a = tc::smem_u32(smem + ONES_OFF);
    const uint32_t b_a = tc::smem_u32(smem + B_OFF);
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

        // ---- prologue (all warps): window luma (+ chroma region), layer 0 ----
        for (int i = tid; i < WW * WH; i += THREADS)
        {
            const int wy = i / WW, wx = i - wy * WW;
            const int gx = clampi(gx0 + wx, 0, W - 1), gy = clampi(gy0 + wy, 0, H - 1);
            const T* src = row_ptr<T>(I.in.ptr, I.in.pitch, gy) + gx * C;
            if constexpr (C == 1) raw[i] = src[0];
            else
            {
                T px[C];
#pragma unroll
                for (int c = 0; c < C; c++) px[c] = src[c];
                T yq, uvq[C - 1];
                rgb_to_yuv_q_lut<T, C>(px, yq, uvq, lut);
                raw[i] = yq;
                const int ux = wx - UVX0, uy = wy - UVX0;
                if (ux >= 0 && ux < UVW && uy >= 0 && uy < UVH)
                {
#pragma unroll
                    for (int c = 0; c < C - 1; c++) uvs[(uy * UVW + ux) * (C - 1) + c] = uvq[c];
                }
            }
        }
        __syncthreads();
        // With chroma the previous tile's horizontal pass left float data in
        // act0, so layer 0 then covers the whole window (its border included).
        constexpr int L0B = C > 1 ? 0 : 1;
        for (int i = tid; i < (WW - 2 * L0B) * (WH - 2 * L0B); i += THREADS)
        {
            const int y = L0B + i / (WW - 2 * L0B), x = L0B + i % (WW - 2 * L0B);
            const int cy = clampi(y, iy0, iy1), cx = clampi(x, ix0, ix1);
            const int ty[3] = {max(cy - 1, iy0), cy, min(cy + 1, iy1)};
            const int tx[3] = {max(cx - 1, ix0), cx, min(cx + 1, ix1)};
            float r[9];
#pragma unroll
            for (int t = 0; t < 9; t++) r[t] = to_float_lut<T>(raw[ty[t / 3] * WW + tx[t % 3]], lut);
            float a[8];
#pragma unroll
            for (int n = 0; n < 8; n++)
            {
                float s = r[0] * P.k0[n * 9];
#pragma unroll
                for (int t = 1; t < 9; t++) s = fmaf(r[t], P.k0[n * 9 + t], s);
                a[n] = s + P.b0[n];
            }
            *slot(act0, y * WW + x) = pack8<BF16>(a);
        }
        tc::fence_proxy_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();

        if (mma_warp)
        {
            if (lane == 0)
            {
                for (int l = 1; l <= NL; l++)
                {
                    const int ry0 = max(l + 1, iy0), ry1 = min(WH - 2 - l, iy1);
                    const int rx0 = max(l + 1, ix0), rx1 = min(WW - 2 - l, ix1);
                    const int b0 = ((ry0 * WW + rx0) >> 1) >> 7, b1 = ((ry1 * WW + rx1) >> 1) >> 7;
                    const uint32_t in_a = ((l - 1) & 1) ? act1_a : act0_a;
                    const uint32_t bl = b_a + static_cast<uint32_t>((l - 1) * BL_BYTES);
                    const uint32_t dbase = tmem + static_cast<uint32_t>((l & 1) * 256);
                    // epilogue counters after layer l-1 of this tile
                    const uint32_t target = 4u * (layers_done + static_cast<uint32_t>(l - 1));
                    for (int b = 0; b < NBLK; b++)
                    {
                        bool ok = true;
                        if (l >= 2)
                            for (int bb = max(0, b - 2); bb <= min(NBLK - 1, b + 2); bb++)
                                ok = ok && wait_count(&epi_cnt[bb], target, abort_flag);
                        tc::fence_after_sync();
                        if (ok && b >= b0 && b <= b1)
                        {
                            const uint32_t d = dbase + static_cast<uint32_t>(b * 16);
#pragma unroll
                            for (int dy = 0; dy < 3; dy++)
                            {
                                const uint32_t a0 = in_a + static_cast<uint32_t>((PADP + b * 128 + (dy - 1) * PPR) * 16);
                                tc::mma_f16(d, tc::smem_desc(a0, PLANE_BYTES - 16, 128),
                                            tc::smem_desc(bl + (2 * dy) * 512, 256, 128), IDESC, dy > 0 ? 1u : 0u);
                                tc::mma_f16(d, tc::smem_desc(a0 + 16, PLANE_BYTES - 16, 128),
                                            tc::smem_desc(bl + (2 * dy + 1) * 512, 256, 128), IDESC, 1u);
                            }
                            tc::mma_f16(d, tc::smem_desc(ones_a, 16, 128), tc::smem_desc(bl + 6 * 512, 256, 128), IDESC, 1u);
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
            for (int l = 1; l <= NL; l++)
            {
                const uint32_t parity = (layers_done + static_cast<uint32_t>(l) - 1u) & 1u;
                const int ry0 = max(l + 1, iy0), ry1 = min(WH - 2 - l, iy1);
                const int rx0 = max(l + 1, ix0), rx1 = min(WW - 2 - l, ix1);
                const int b0 = ((ry0 * WW + rx0) >> 1) >> 7, b1 = ((ry1 * WW + rx1) >> 1) >> 7;
                unsigned char* out_act = (l & 1) ? act1 : act0;
                float* Hs = reinterpret_cast<float*>(act0);  // last layer: act0 held layer 6, free once layer 8 runs
                if constexpr (C > 1)
                {
                    if (l == NL)
                    {
                        // the horizontal chroma pass once MMA(8, block 0) completed (so all
                        // layer-7 MMAs, the last readers of act0, completed too)
                        const bool ok = __all_sync(0xffffffffu, wait_bar(&mma_bar[0], parity, abort_flag) ? 1 : 0);
                        if (ok)
                            for (int e = tid; e < UVH * 2 * TW; e += NEPI * 32)
                            {
                                const int r = e / (2 * TW), ox = e - r * (2 * TW);
                                chroma_hpass<T, C - 1>(uvs + r * UVW * (C - 1), ox >> 1, ox & 1, P.ph, Hs + e * (C - 1));
                            }
                        // bounded barrier of the sixteen epilogue warps
                        __syncwarp();
                        gbar_gen++;
                        if (lane == 0) tc::smem_add_release(gbar, 1);
                        wait_count(gbar, NEPI * gbar_gen, abort_flag);
                        __syncwarp();
                    }
                }
                for (int b = g; b < NBLK; b += 4)
                {
                    const bool done = __all_sync(0xffffffffu, wait_bar(&mma_bar[b], parity, abort_flag) ? 1 : 0);
                    tc::fence_after_sync();
                    if (done && b >= b0 && b <= b1)
                    {
                        float v[16];
                        tc::tmem_ld16(tmem + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>((l & 1) * 256 + b * 16), v);
                        tc::tmem_wait_ld();
                        const int r = b * 128 + q * 32 + lane;
#pragma unroll
                        for (int k = 0; k < 2; k++)
                        {
                            const int p = 2 * r + k;
                            const int y = p / WW, x = p - y * WW;
                            if (y < ry0 || y > ry1 || x < rx0 || x > rx1) continue;
                            if (l < NL)
                            {
                                const uint4 val = pack8<BF16>(v + 8 * k);
                                *slot(out_act, p) = val;
                                const bool xl = x == ix0 && x > 0, xr = x == ix1 && x < WW - 1;
                                const bool yt = y == iy0 && y > 0, yb = y == iy1 && y < WH - 1;
                                if (xl) *slot(out_act, p - 1) = val;
                                if (xr) *slot(out_act, p + 1) = val;
                                if (yt)
                                {
                                    *slot(out_act, p - WW) = val;
                                    if (xl) *slot(out_act, p - WW - 1) = val;
                                    if (xr) *slot(out_act, p - WW + 1) = val;
                                }
                                if (yb)
                                {
                                    *slot(out_act, p + WW) = val;
                                    if (xl) *slot(out_act, p + WW - 1) = val;
                                    if (xr) *slot(out_act, p + WW + 1) = val;
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
                                        for (int c = 1; c < 8; c++) d = fmaf(s[c], P.k2[ko + c], d);
                                        o[dy][dx] = from_float<T>(d);
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
                                else merge_block2_h<T, C>(Hs, 2 * TW, x - HALO, y - HALO, P.ph, o, row0, row1, lut);
                            }
                        }
                    }
                    // publish: activations visible to the tensor core, tensor-memory reads done
                    tc::fence_proxy_async_smem();
                    tc::fence_before_sync();
                    __syncwarp();
                    if (lane == 0) tc::smem_add_release(&epi_cnt[b], 1);
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

template <typename T, int C, bool BF16>
cudaError_t launch_typed(const Params& p, int grid, cudaStream_t stream)
{
    static bool configured = false;
    if (!configured)
    {
        cudaError_t err = cudaFuncSetAttribute(acnet_tc3_kernel<T, C, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               Layout<T, C>::smem);
        if (err != cudaSuccess) return err;
        configured = true;
    }
    acnet_tc3_kernel<T, C, BF16><<<grid, THREADS, Layout<T, C>::smem, stream>>>(p);
    return cudaGetLastError();
}

template <typename T, bool BF16>
cudaError_t launch_channels(int c, const Params& p, int grid, cudaStream_t stream)
{
    switch (c)
    {
    case 1: return launch_typed<T, 1, BF16>(p, grid, stream);
    case 3: return launch_typed<T, 3, BF16>(p, grid, stream);
    case 4: return launch_typed<T, 4, BF16>(p, grid, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace tcv3

int* tc_status_buffer();

int acnet_tc3_max_images() { return tcv3::kMaxImages; }

// One persistent launch over all tiles of n images (same element type and
// channel count; each output exactly 2x its input).  `counter` is a device
// int the call zeroes on `stream` before the launch; `ctas` CTAs (one per SM
// at most is resident) drain the queue.
cudaError_t launch_acnet_legacy_tc3(const AcnetLegacyWeights& wts, const void* packed2, bool bf16, int n, const Plane* in,
                                    const Plane* out, const Phase2* phase2, int* counter, int ctas, cudaStream_t stream)
{
    using namespace tcv3;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxImages || !packed2 || !counter) return cudaErrorInvalidValue;
    const int c = in[0].channels, type = in[0].type;
    if (c > 1 && !phase2) return cudaErrorInvalidValue;
    Params p;
    std::memset(&p, 0, sizeof(p));
    p.bw = static_cast<const uint4*>(packed2);
    for (int i = 0; i < 72; i++) p.k0[i] = wts.k[i];
    for (int i = 0; i < 8; i++) p.b0[i] = wts.b[i];
    for (int i = 0; i < 32; i++) p.k2[i] = wts.k[72 + 576 * 8 + i];
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
    p.status = tc_status_buffer();
    if (!p.status) return cudaErrorMemoryAllocation;
    cudaError_t err = cudaMemsetAsync(counter, 0, sizeof(int), stream);
    if (err != cudaSuccess) return err;
    const int grid = tiles < ctas ? tiles : ctas;
    switch (type)
    {
    case kU8: err = bf16 ? launch_channels<uint8_t, true>(c, p, grid, stream) : launch_channels<uint8_t, false>(c, p, grid, stream); break;
    case kU16: err = bf16 ? launch_channels<uint16_t, true>(c, p, grid, stream) : launch_channels<uint16_t, false>(c, p, grid, stream); break;
    case kF32: err = bf16 ? launch_channels<float, true>(c, p, grid, stream) : launch_channels<float, false>(c, p, grid, stream); break;
    default: return cudaErrorInvalidValue;
    }
    if (err == cudaSuccess) count_launch();
    return err;
}

}  // namespace acgb
