// ArtCNN<16/32> and FSRCNNX<16> x2 passes in a tensor-core form (FP16 or BF16
// operands, FP32 accumulation): the 3x3 F->F layers and the F->4 upscale on
// tcgen05, the 1->F head in FP32 on CUDA cores, F-channel 16-bit maps between
// launches.
//
// Networks and CPU order as k_f3_fp32.cu (CPUProcessor.cpp:1519-1600,
// 1629-1715).  GEMM shape: one GEMM row = one pixel, N = F output channels,
// K = 9 taps x F input channels.  A window of 32 x 32 pixels (halo 1 around a
// 30 x 30 tile) is held as F/8 channel planes (16 bytes = 8 channels per
// pixel each); for tap (dy, dx) and channels 16 j .. 16 j + 15 the A operand
// is a shifted view of planes 2 j and 2 j + 1 (leading byte offset = one
// plane), so a tap is F/16 M128 x N F x K16 MMAs and a block of 128 pixels
// 9 F/16 of them.  8 blocks per window, F tensor-memory columns each.
//
// Two kernels run these GEMMs: convw_kernel, one CTA per tile (the 16-channel
// 3x3 layers but FSRCNNX's tail), and convp_kernel, persistent CTAs with a
// TMA-fed two-stage pipeline (the 32-channel layers, FSRCNNX's tail, whose
// FP32 1x1 epilogue it overlaps with the MMAs, and every upscale layer, which
// it runs with N = 16 and the weights split into 16-bit high parts and
// residuals).
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "kernels.hpp"
#include "tc_ptx.cuh"
#include "tma_host.hpp"

namespace acgb {
namespace f3tc {

constexpr int WW = 32, WH = 32, TW = WW - 2, TH = WH - 2;
constexpr int NBLK = WW * WH / 128;  // 8
constexpr int PAD = 40;              // >= WW + 1: taps of the first and last rows stay inside a plane
constexpr int PLANE_BYTES = (PAD + NBLK * 128 + PAD) * 16;
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr int kMaxImg = 16;

enum Mode { kReLU = 0, kPReLU = 1, kAddSkip = 2, kFsrTail = 3, kUp = 4 };

template <int F>
struct Geo
{
    static constexpr int NP = F / 8;                  // channel planes
    static constexpr int CHUNK = F * 32;              // B of one MMA: N F x K16 x 16 bit
    static constexpr int B_BYTES = 9 * (F / 16) * CHUNK;
    static constexpr uint32_t TMEM_COLS = NBLK * F;   // 128 (F = 16) or 256 (F = 32)
    static constexpr int SMEM = NP * PLANE_BYTES + B_BYTES + 64;
    // at most 512 / TMEM_COLS CTAs per SM: request enough shared memory to enforce it
    static constexpr int MIN_SMEM = (228 * 1024) / (512 / TMEM_COLS + 1) + 1024;
    static constexpr int SMEM_REQ = SMEM > MIN_SMEM ? SMEM : MIN_SMEM;
    // 1,024 threads per SM over the CTAs that fit (2 for F = 32, 4 for F = 16):
    // many window loads in flight, several warps per tensor-memory lane quarter
    static constexpr int THREADS = F == 32 ? 512 : 256;
};

struct ImgW
{
    const uint4* in;    // [h][w] pixels of F 16-bit channels
    uint4* out;
    const uint4* skip;  // kAddSkip: the map added; kFsrTail: feat
    int w, h, tiles_x, tile0;
};

template <int F>
struct ConvWP
{
    const uint4* bw;  // packed B (pack_f3_conv)
    float b[F], a[F];
    float k1[F * F], b1[F], a1[F];  // kFsrTail: conv1x1 F->F, bias, PReLU
    int* status;
    int nimg;
    ImgW img[kMaxImg];
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
            const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&r[i]));
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

template <int F, int MODE, bool BF16>
__global__ void __launch_bounds__(Geo<F>::THREADS) convw_kernel(const __grid_constant__ ConvWP<F> P)
{
    using G = Geo<F>;
    constexpr int THREADS = G::THREADS;
    constexpr int NP = G::NP;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* planes = smem;
    unsigned char* bsm = smem + NP * PLANE_BYTES;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(bsm + G::B_BYTES);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bsm + G::B_BYTES + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int im = 0;
    while (im + 1 < P.nimg && P.img[im + 1].tile0 <= static_cast<int>(blockIdx.x)) im++;
    const ImgW& I = P.img[im];
    const int local = static_cast<int>(blockIdx.x) - I.tile0;
    const int x0 = (local % I.tiles_x) * TW - 1, y0 = (local / I.tiles_x) * TH - 1;

    if (tid == 0)
    {
        tc::mbar_init(mbar, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0)
    {
        tc::tmem_alloc(tmem_slot, G::TMEM_COLS);
        tc::tmem_relinquish();
    }
    for (int i = tid; i < G::B_BYTES / 16; i += THREADS) reinterpret_cast<uint4*>(bsm)[i] = P.bw[i];
    // pads: read with zero weights by the window's first and last rows
    for (int i = tid; i < NP * 2 * PAD; i += THREADS)
    {
        const int pl = i / (2 * PAD), k = i % (2 * PAD);
        reinterpret_cast<uint4*>(planes + pl * PLANE_BYTES)[k < PAD ? k : NBLK * 128 + k] = make_uint4(0, 0, 0, 0);
    }
    // the window (clamped to the map): pixel p's channels 8 j .. 8 j + 7 into
    // plane j, four loads in flight per thread
    constexpr int NLD = WW * WH * NP / THREADS;
    static_assert(NLD % 4 == 0 && NLD * THREADS == WW * WH * NP, "whole load batches");
#pragma unroll 1
    for (int k0 = 0; k0 < NLD; k0 += 4)
    {
        uint4 v[4];
        int dst[4];
#pragma unroll
        for (int k = 0; k < 4; k++)
        {
            const int i = tid + (k0 + k) * THREADS;
            const int p = i / NP, j = i - p * NP;
            const int wy = p / WW, wx = p - wy * WW;
            const int gx = clampi(x0 + wx, 0, I.w - 1), gy = clampi(y0 + wy, 0, I.h - 1);
            v[k] = I.in[(static_cast<size_t>(gy) * I.w + gx) * NP + j];
            dst[k] = j * (PLANE_BYTES / 16) + PAD + p;
        }
#pragma unroll
        for (int k = 0; k < 4; k++) reinterpret_cast<uint4*>(planes)[dst[k]] = v[k];
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    if (tid == 0)
    {
        constexpr uint32_t IDESC = tc::idesc_f16(128, F, BF16);
        const uint32_t pl0 = tc::smem_u32(planes), b0 = tc::smem_u32(bsm);
        for (int b = 0; b < NBLK; b++)
        {
#pragma unroll
            for (int t = 0; t < 9; t++)
            {
                const int slot = PAD + 128 * b + (t / 3 - 1) * WW + (t % 3 - 1);
#pragma unroll
                for (int j2 = 0; j2 < F / 16; j2++)
                {
                    const uint64_t a = tc::smem_desc(pl0 + static_cast<uint32_t>(2 * j2 * PLANE_BYTES + slot * 16), PLANE_BYTES, 128);
                    const uint64_t bd =
                        tc::smem_desc(b0 + static_cast<uint32_t>((t * (F / 16) + j2) * G::CHUNK), F * 16, 128);
                    tc::mma_f16(tmem + static_cast<uint32_t>(b * F), a, bd, IDESC, (t | j2) ? 1u : 0u);
                }
            }
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
        // warp w drains lane quarter w % 4 of blocks w / 4, w / 4 + THREADS / 128, ...
        for (int b = warp >> 2; b < NBLK; b += THREADS / 128)
        {
            const int q4 = warp & 3;
            float v[F];
#pragma unroll
            for (int h = 0; h < F / 16; h++)
            {
                float q[16];
                tc::tmem_ld16(tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>(b * F + 16 * h), q);
                tc::tmem_wait_ld();
#pragma unroll
                for (int c = 0; c < 16; c++) v[16 * h + c] = q[c];
            }
            const int p = b * 128 + q4 * 32 + lane;
            const int y = p / WW, x = p - y * WW;
            const int gx = x0 + x, gy = y0 + y;
            if (y < 1 || y > TH || x < 1 || x > TW || gx >= I.w || gy >= I.h) continue;
            const size_t o = (static_cast<size_t>(gy) * I.w + gx) * NP;
#pragma unroll
            for (int n = 0; n < F; n++) v[n] += P.b[n];
            if constexpr (MODE == kReLU)
            {
#pragma unroll
                for (int n = 0; n < F; n++) v[n] = fmaxf(v[n], 0.0f);
            }
            else if constexpr (MODE == kPReLU || MODE == kFsrTail)
            {
#pragma unroll
                for (int n = 0; n < F; n++) v[n] = prelu(v[n], P.a[n]);
            }
            if constexpr (MODE == kAddSkip)
            {
#pragma unroll
                for (int j = 0; j < NP; j++)
                {
                    float sk[8];
                    unpack8<BF16>(I.skip[o + j], sk);
#pragma unroll
                    for (int c = 0; c < 8; c++) v[8 * j + c] += sk[c];
                }
            }
            if constexpr (MODE == kFsrTail)
            {
                // conv1x1 F->F + bias, + feat, PReLU
                float u[F];
#pragma unroll
                for (int n = 0; n < F; n++)
                {
                    float s = P.b1[n];
#pragma unroll
                    for (int c = 0; c < F; c++) s = fmaf(v[c], P.k1[n * F + c], s);
                    u[n] = s;
                }
#pragma unroll
                for (int j = 0; j < NP; j++)
                {
                    float f[8];
                    unpack8<BF16>(I.skip[o + j], f);
#pragma unroll
                    for (int c = 0; c < 8; c++) v[8 * j + c] = prelu(u[8 * j + c] + f[c], P.a1[8 * j + c]);
                }
            }
#pragma unroll
            for (int j = 0; j < NP; j++) I.out[o + j] = pack8<BF16>(v + 8 * j);
        }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, G::TMEM_COLS);
}

// ---- persistent form ----
// One CTA per SM (F = 32) or two (F = 16) walk the tiles of a layer with a
// two-stage pipeline: while the epilogue warps drain tile t's accumulators,
// the MMA lane runs tile t + 1 and the producer warp loads tile t + 2's window
// with TMA (one 8 x 32 x 32 box per channel plane; the out-of-image ring that
// clamp-to-edge needs is then copied in from its neighbours).  Stage s of
// tile t (s = t % 2, u = t / 2):
//   full[s]   TMA bytes of the window landed          (producer waits)
//   ready[s]  window complete, edge ring filled       (MMA lane waits)
//   mdone[s]  MMAs of the stage completed (commit)    (epilogue, producer wait)
//   tfree[s]  accumulators drained by every epilogue warp (MMA lane waits)
// Each wait targets completion u (or u - 1) of a barrier whose next completion
// needs the waiter's own progress, so no phase is ever skipped.  Every wait is
// bounded; a timeout raises the CTA's abort flag and the status word.
constexpr int NSTAGE = 2;

template <int F>
struct GeoP
{
    static constexpr int NP = F / 8;
    static constexpr int WIN_BYTES = NP * PLANE_BYTES;
    static constexpr int CHUNK = F * 32;
    static constexpr int B_BYTES = 9 * (F / 16) * CHUNK;
    static constexpr uint32_t TMEM_COLS = NSTAGE * NBLK * F;  // 256 (F = 16) or 512 (F = 32)
    static constexpr int NEPI = F == 32 ? 16 : 8;            // epilogue warps, a multiple of 4
    static constexpr int THREADS = (2 + NEPI) * 32;
    static constexpr int MINB = F == 32 ? 1 : 2;             // CTAs per SM
    static constexpr int BAR_OFF = NSTAGE * WIN_BYTES + B_BYTES;
    static constexpr int SMEM = BAR_OFF + 128;
    // at most 512 / TMEM_COLS CTAs per SM: request enough shared memory to enforce it
    static constexpr int MIN_SMEM = (228 * 1024) / (512 / TMEM_COLS + 1) + 1024;
    static constexpr int SMEM_REQ = SMEM > MIN_SMEM ? SMEM : MIN_SMEM;
    static constexpr uint32_t BOX_BYTES = 8 * WW * WH * 2;  // one channel plane of the window
    static_assert((PAD * 16) % 128 == 0 && PLANE_BYTES % 128 == 0, "TMA destinations 128-byte aligned");
};

struct ImgP
{
    const uint4* skip;  // kAddSkip: the map added; kFsrTail: feat
    uint4* out;
    int w, h, tiles_x, tile0;
    Plane dst;  // kUp: the 2w x 2h output plane
};

template <int F>
struct ConvPP
{
    CUtensorMap tmap[kMaxImg];  // input map of each image: [h][w][F] 16-bit, box 8 x 32 x 32
    const uint4* bw;            // packed B (pack_f3_conv)
    float b[F], a[F];
    float k1[F * F], b1[F], a1[F];  // kFsrTail: conv1x1 F->F, bias, PReLU
    int* status;
    int nimg, ntiles;
    ImgP img[kMaxImg];
};

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

template <int F>
__device__ __forceinline__ int image_of(const ConvPP<F>& P, int tile)
{
    int im = 0;
    while (im + 1 < P.nimg && P.img[im + 1].tile0 <= tile) im++;
    return im;
}

// MODE kUp: the F -> 4 upscale layer with N = 16 (columns 0-3 the weights'
// 16-bit high parts, 4-7 their residuals), pixel shuffle into the OT plane.
template <int F, int MODE, bool BF16, typename OT>
__global__ void __launch_bounds__(GeoP<F>::THREADS, GeoP<F>::MINB) convp_kernel(const __grid_constant__ ConvPP<F> P)
{
    using G = GeoP<F>;
    constexpr int NP = G::NP, NEPI = G::NEPI;
    constexpr int NM = MODE == kUp ? 16 : F;           // MMA N
    constexpr int CHUNK_M = NM * 32;                   // B of one MMA
    constexpr int BB = 9 * (F / 16) * CHUNK_M;         // this layer's B
    static_assert(BB <= G::B_BYTES, "B fits its buffer");
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* bsm = smem + NSTAGE * G::WIN_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + G::BAR_OFF);
    uint64_t* full = bars;       // [NSTAGE]
    uint64_t* ready = bars + 2;  // [NSTAGE]
    uint64_t* mdone = bars + 4;  // [NSTAGE]
    uint64_t* tfree = bars + 6;  // [NSTAGE]
    uint64_t* bbar = bars + 8;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 9);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 10);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

    if (tid == 0)
    {
        for (int i = 0; i < NSTAGE; i++)
        {
            tc::mbar_init(&full[i], 1);
            tc::mbar_init(&ready[i], 1);
            tc::mbar_init(&mdone[i], 1);
            tc::mbar_init(&tfree[i], NEPI);
        }
        tc::mbar_init(bbar, 1);
        *abort_flag = 0;
        tc::fence_mbar_init();
    }
    // the planes' pads (never loaded): read with zero weights by the window's first and last rows
    for (int i = tid; i < NSTAGE * NP * 2 * PAD; i += G::THREADS)
    {
        const int pl = i / (2 * PAD), k = i % (2 * PAD);
        reinterpret_cast<uint4*>(smem + pl * PLANE_BYTES)[k < PAD ? k : NBLK * 128 + k] = make_uint4(0, 0, 0, 0);
    }
    if (warp == 1)
    {
        tc::tmem_alloc(tmem_slot, G::TMEM_COLS);
        tc::tmem_relinquish();
    }
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0)
    {
        // ---- producer ----
        if (lane == 0)
        {
            tc::mbar_arrive_expect_tx(bbar, BB);
            tc::bulk_load(bsm, P.bw, BB, bbar);
        }
        int it = 0;
        bool pending = false;  // a window load issued and not yet seen complete
        for (int tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x, it++)
        {
            const int s = it & 1;
            const uint32_t u = static_cast<uint32_t>(it) >> 1;
            bool ok = u == 0 || wait_bar(&mdone[s], (u - 1) & 1u, abort_flag);
            if (!__all_sync(0xffffffffu, ok ? 1 : 0)) break;
            const int im = image_of(P, tile);
            const ImgP& I = P.img[im];
            const int local = tile - I.tile0;
            const int x0 = (local % I.tiles_x) * TW - 1, y0 = (local / I.tiles_x) * TH - 1;
            unsigned char* win = smem + s * G::WIN_BYTES;
            if (lane == 0)
            {
                tc::mbar_arrive_expect_tx(&full[s], NP * G::BOX_BYTES);
#pragma unroll
                for (int j = 0; j < NP; j++) tc::tma_load_3d(win + j * PLANE_BYTES + PAD * 16, &P.tmap[im], 8 * j, x0, y0, &full[s]);
            }
            pending = true;
            ok = wait_bar(&full[s], u & 1u, abort_flag);
            if (!__all_sync(0xffffffffu, ok ? 1 : 0)) break;
            pending = false;
            // clamp-to-edge: the window column / row just outside the image
            // takes its inner neighbour (columns first, so corners follow)
            const int xl = x0 < 0 ? 0 : -1, xr = I.w - x0 < WW ? I.w - x0 : -1;
            const int yt = y0 < 0 ? 0 : -1, yb = I.h - y0 < WH ? I.h - y0 : -1;
            if (xl >= 0 || xr >= 0 || yt >= 0 || yb >= 0)
            {
                uint4* pw = reinterpret_cast<uint4*>(win) + PAD;
                for (int i = lane; i < WH * NP; i += 32)
                {
                    uint4* row = pw + (i % NP) * (PLANE_BYTES / 16) + (i / NP) * WW;
                    if (xl >= 0) row[xl] = row[xl + 1];
                    if (xr >= 0) row[xr] = row[xr - 1];
                }
                __syncwarp();
                for (int i = lane; i < WW * NP; i += 32)
                {
                    uint4* col = pw + (i % NP) * (PLANE_BYTES / 16) + i / NP;
                    if (yt >= 0) col[yt * WW] = col[(yt + 1) * WW];
                    if (yb >= 0) col[yb * WW] = col[(yb - 1) * WW];
                }
                tc::fence_proxy_async_smem();
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&ready[s]);
        }
        // loads still in flight (after an abort) land before the CTA exits;
        // bounded by time, not cut short by the abort
        if (lane == 0)
        {
            if (pending && !tc::mbar_wait_ns(&full[it & 1], (static_cast<uint32_t>(it) >> 1) & 1u, kWaitNs)) *abort_flag = 1;
            if (!tc::mbar_wait_ns(bbar, 0, kWaitNs)) *abort_flag = 1;
        }
        __syncwarp();
    }
    else if (warp == 1)
    {
        // ---- MMA issue ----
        if (lane == 0)
        {
            constexpr uint32_t IDESC = tc::idesc_f16(128, NM, BF16);
            const uint32_t b0 = tc::smem_u32(bsm);
            bool ok = wait_bar(bbar, 0, abort_flag);
            int it = 0, last = -1;
            for (int tile = blockIdx.x; ok && tile < P.ntiles; tile += gridDim.x, it++)
            {
                const int s = it & 1;
                const uint32_t u = static_cast<uint32_t>(it) >> 1;
                ok = wait_bar(&ready[s], u & 1u, abort_flag);
                if (ok && u >= 1) ok = wait_bar(&tfree[s], (u - 1) & 1u, abort_flag);
                if (!ok) break;
                tc::fence_after_sync();
                // descriptors: stage s plane 0 slot 0 and B chunk 0, then
                // compile-time offsets in 16-byte units per tap and channel pair
                const uint64_t adesc = tc::smem_desc(tc::smem_u32(smem + s * G::WIN_BYTES), PLANE_BYTES, 128);
                const uint64_t bdesc = tc::smem_desc(b0, NM * 16, 128);
#pragma unroll 1
                for (int b = 0; b < NBLK; b++)
                {
                    const uint32_t d = tmem + static_cast<uint32_t>((s * NBLK + b) * F);
                    const uint64_t ab = adesc + static_cast<uint64_t>(PAD + 128 * b);
#pragma unroll
                    for (int t = 0; t < 9; t++)
#pragma unroll
                        for (int j2 = 0; j2 < F / 16; j2++)
                        {
                            constexpr int PL16 = PLANE_BYTES / 16;
                            const int off = 2 * j2 * PL16 + (t / 3 - 1) * WW + (t % 3 - 1);
                            tc::mma_f16(d, ab + static_cast<uint64_t>(static_cast<int64_t>(off)),
                                        bdesc + static_cast<uint64_t>((t * (F / 16) + j2) * (CHUNK_M / 16)), IDESC,
                                        (t | j2) ? 1u : 0u);
                        }
                }
                tc::mma_commit(&mdone[s]);
                last = it;
            }
            // the last MMAs complete before tensor memory is released
            if (last >= 0 && !tc::mbar_wait_ns(&mdone[last & 1], (static_cast<uint32_t>(last) >> 1) & 1u, kWaitNs))
                *abort_flag = 1;
        }
        __syncwarp();
    }
    else
    {
        // ---- epilogue: warp w drains lane quarter w % 4 of blocks (w - 2) / 4 + k NEPI / 4 ----
        const int q4 = warp & 3, part = (warp - 2) >> 2;
        int it = 0;
        for (int tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x, it++)
        {
            const int s = it & 1;
            const uint32_t u = static_cast<uint32_t>(it) >> 1;
            const bool got = wait_bar(&mdone[s], u & 1u, abort_flag);
            if (!__all_sync(0xffffffffu, got ? 1 : 0)) break;
            tc::fence_after_sync();
            const ImgP& I = P.img[image_of(P, tile)];
            const int local = tile - I.tile0;
            const int x0 = (local % I.tiles_x) * TW - 1, y0 = (local / I.tiles_x) * TH - 1;
            for (int b = part; b < NBLK; b += NEPI / 4)
            {
                if constexpr (MODE == kUp)
                {
                    float q[16];
                    tc::tmem_ld16(tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>((s * NBLK + b) * F), q);
                    tc::tmem_wait_ld();
                    const int p = b * 128 + q4 * 32 + lane;
                    const int y = p / WW, x = p - y * WW;
                    const int gx = x0 + x, gy = y0 + y;
                    if (y < 1 || y > TH || x < 1 || x > TW || gx >= I.w || gy >= I.h) continue;
                    // conv3x3 F -> 4 + bias, pixel shuffle 2x2, fromFloat (no nearest add)
                    OT* r0 = row_ptr_w<OT>(I.dst.ptr, I.dst.pitch, 2 * gy) + 2 * gx;
                    OT* r1 = row_ptr_w<OT>(I.dst.ptr, I.dst.pitch, 2 * gy + 1) + 2 * gx;
                    r0[0] = from_float<OT>(q[0] + q[4] + P.b[0]);
                    r0[1] = from_float<OT>(q[1] + q[5] + P.b[1]);
                    r1[0] = from_float<OT>(q[2] + q[6] + P.b[2]);
                    r1[1] = from_float<OT>(q[3] + q[7] + P.b[3]);
                    continue;
                }
                float v[F];
#pragma unroll
                for (int h = 0; h < F / 16; h++)
                {
                    float q[16];
                    tc::tmem_ld16(tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>((s * NBLK + b) * F + 16 * h), q);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int c = 0; c < 16; c++) v[16 * h + c] = q[c];
                }
                const int p = b * 128 + q4 * 32 + lane;
                const int y = p / WW, x = p - y * WW;
                const int gx = x0 + x, gy = y0 + y;
                if (y < 1 || y > TH || x < 1 || x > TW || gx >= I.w || gy >= I.h) continue;
                const size_t o = (static_cast<size_t>(gy) * I.w + gx) * NP;
#pragma unroll
                for (int n = 0; n < F; n++) v[n] += P.b[n];
                if constexpr (MODE == kReLU)
                {
#pragma unroll
                    for (int n = 0; n < F; n++) v[n] = fmaxf(v[n], 0.0f);
                }
                else if constexpr (MODE == kPReLU || MODE == kFsrTail)
                {
#pragma unroll
                    for (int n = 0; n < F; n++) v[n] = prelu(v[n], P.a[n]);
                }
                if constexpr (MODE == kAddSkip)
                {
#pragma unroll
                    for (int j = 0; j < NP; j++)
                    {
                        float sk[8];
                        unpack8<BF16>(I.skip[o + j], sk);
#pragma unroll
                        for (int c = 0; c < 8; c++) v[8 * j + c] += sk[c];
                    }
                }
                if constexpr (MODE == kFsrTail)
                {
                    // conv1x1 F->F + bias, + feat, PReLU
                    float uo[F];
#pragma unroll
                    for (int n = 0; n < F; n++)
                    {
                        float a1 = P.b1[n];
#pragma unroll
                        for (int c = 0; c < F; c++) a1 = fmaf(v[c], P.k1[n * F + c], a1);
                        uo[n] = a1;
                    }
#pragma unroll
                    for (int j = 0; j < NP; j++)
                    {
                        float f[8];
                        unpack8<BF16>(I.skip[o + j], f);
#pragma unroll
                        for (int c = 0; c < 8; c++) v[8 * j + c] = prelu(uo[8 * j + c] + f[c], P.a1[8 * j + c]);
                    }
                }
#pragma unroll
                for (int j = 0; j < NP; j++) I.out[o + j] = pack8<BF16>(v + 8 * j);
            }
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&tfree[s]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    if (tid == 0 && *abort_flag) atomicExch(P.status, 1);
    if (warp == 1) tc::tmem_dealloc(tmem, G::TMEM_COLS);
}

template <int K, int F>
struct HeadP
{
    float k[F * K * K];
    float b[F];
};

// conv KxK 1 -> F (identity) in FP32 from the input plane, taps clamped,
// stored as an F-channel 16-bit map.
template <typename T, int K, int F, bool BF16>
__global__ void __launch_bounds__(256) head_kernel(const __grid_constant__ HeadP<K, F> W, Plane in, uint4* __restrict__ feat)
{
    constexpr int R = K / 2, SW = 32 + 2 * R, SH = 8 + 2 * R;
    // the block's 32 x 8 pixels with their clamped halo, converted once
    __shared__ float s[SH][SW];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 8;
    for (int i = threadIdx.x; i < SW * SH; i += 256)
    {
        const int sy = i / SW, sx = i - sy * SW;
        const int gx = clampi(bx - R + sx, 0, in.w - 1), gy = clampi(by - R + sy, 0, in.h - 1);
        s[sy][sx] = to_float<T>(row_ptr<T>(in.ptr, in.pitch, gy)[gx]);
    }
    __syncthreads();
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int x = bx + tx, y = by + ty;
    if (x >= in.w || y >= in.h) return;
    float t[K * K];
#pragma unroll
    for (int p = 0; p < K * K; p++) t[p] = s[ty + p / K][tx + p % K];
    uint4* o = feat + (static_cast<size_t>(y) * in.w + x) * (F / 8);
#pragma unroll
    for (int j = 0; j < F / 8; j++)
    {
        float r[8];
#pragma unroll
        for (int c = 0; c < 8; c++)
        {
            float v = W.b[8 * j + c];
#pragma unroll
            for (int p = 0; p < K * K; p++) v = fmaf(t[p], W.k[(8 * j + c) * K * K + p], v);
            r[c] = v;
        }
        o[j] = pack8<BF16>(r);
    }
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

// One 3x3 F->F layer k[n * 9F + tap * F + c] as the 9 F/16 B chunks of the
// GEMM: chunk (tap t, channel pair j2) element (n, kk) = k[n][t][16 j2 + kk]
// at byte (kk / 8) 16F + (n / 8) 128 + (n % 8) 16 + (kk % 8) 2.
void pack_f3_conv(const float* k, int F, bool bf16, uint16_t* out)
{
    const int chunk = F * 32;
    std::memset(out, 0, static_cast<size_t>(9) * (F / 16) * chunk);
    for (int t = 0; t < 9; t++)
        for (int j2 = 0; j2 < F / 16; j2++)
        {
            uint16_t* ch = out + (t * (F / 16) + j2) * (chunk / 2);
            for (int n = 0; n < F; n++)
                for (int kk = 0; kk < 16; kk++)
                    ch[((kk >> 3) * 16 * F + (n >> 3) * 128 + (n & 7) * 16 + (kk & 7) * 2) / 2] =
                        to_bits(k[n * 9 * F + t * F + 16 * j2 + kk], bf16);
        }
}

float from_bits(uint16_t b, bool bf16)
{
    if (bf16)
    {
        const uint32_t u = static_cast<uint32_t>(b) << 16;
        float v;
        std::memcpy(&v, &u, 4);
        return v;
    }
    return __half2float(__ushort_as_half(b));
}

// The upscale layer k[n * 9F + tap * F + c] (n < 4) as the 9 F/16 B chunks of
// an N = 16 GEMM: column n < 4 holds the 16-bit weight, column n + 4 the
// 16-bit residual w - hi (together exact to about 2^-22), columns 8..15 zero.
// Chunk (tap t, channel pair j2) element (n, kk) at byte
// (kk / 8) 256 + (n / 8) 128 + (n % 8) 16 + (kk % 8) 2.
void pack_f3_up(const float* k, int F, bool bf16, uint16_t* out)
{
    constexpr int N = 16;
    std::memset(out, 0, static_cast<size_t>(9) * F * N * 2);
    for (int t = 0; t < 9; t++)
        for (int j2 = 0; j2 < F / 16; j2++)
        {
            uint16_t* ch = out + (t * (F / 16) + j2) * (N * 16);
            for (int n = 0; n < 8; n++)
                for (int kk = 0; kk < 16; kk++)
                {
                    const float wv = k[(n & 3) * 9 * F + t * F + 16 * j2 + kk];
                    const uint16_t hi = to_bits(wv, bf16);
                    ch[((kk >> 3) * 16 * N + (n >> 3) * 128 + (n & 7) * 16 + (kk & 7) * 2) / 2] =
                        n < 4 ? hi : to_bits(wv - from_bits(hi, bf16), bf16);
                }
        }
}

template <int F, int MODE, bool BF16>
cudaError_t launch_conv(const ConvWP<F>& p, int tiles, cudaStream_t stream)
{
    using G = Geo<F>;
    static bool configured = false;
    if (!configured)
    {
        cudaError_t err = cudaFuncSetAttribute(convw_kernel<F, MODE, BF16>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM_REQ);
        if (err != cudaSuccess) return err;
        configured = true;
    }
    convw_kernel<F, MODE, BF16><<<tiles, G::THREADS, G::SMEM_REQ, stream>>>(p);
    return cudaGetLastError();
}

template <int F, int MODE, bool BF16, typename OT = uint8_t>
cudaError_t launch_convp(const ConvPP<F>& p, cudaStream_t stream)
{
    using G = GeoP<F>;
    static int per_sm = 0, sms = 0;
    if (per_sm == 0)
    {
        cudaError_t err =
            cudaFuncSetAttribute(convp_kernel<F, MODE, BF16, OT>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM_REQ);
        if (err != cudaSuccess) return err;
        int occ = 0, dev = 0;
        if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, convp_kernel<F, MODE, BF16, OT>, G::THREADS, G::SMEM_REQ)) !=
            cudaSuccess)
            return err;
        if ((err = cudaGetDevice(&dev)) != cudaSuccess) return err;
        if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return err;
        if (occ < 1) return cudaErrorInvalidConfiguration;
        per_sm = occ < static_cast<int>(512 / G::TMEM_COLS) ? occ : static_cast<int>(512 / G::TMEM_COLS);
    }
    const int grid = p.ntiles < per_sm * sms ? p.ntiles : per_sm * sms;
    convp_kernel<F, MODE, BF16, OT><<<grid, G::THREADS, G::SMEM_REQ, stream>>>(p);
    return cudaGetLastError();
}

template <int F, bool BF16>
cudaError_t convp_mode(int mode, const ConvPP<F>& p, cudaStream_t stream)
{
    switch (mode)
    {
    case kReLU: return launch_convp<F, kReLU, BF16>(p, stream);
    case kPReLU: return launch_convp<F, kPReLU, BF16>(p, stream);
    case kAddSkip: return launch_convp<F, kAddSkip, BF16>(p, stream);
    default: return launch_convp<F, kFsrTail, BF16>(p, stream);
    }
}

template <int F, bool BF16>
cudaError_t conv_mode(int mode, const ConvWP<F>& p, int tiles, cudaStream_t stream)
{
    switch (mode)
    {
    case kReLU: return launch_conv<F, kReLU, BF16>(p, tiles, stream);
    case kPReLU: return launch_conv<F, kPReLU, BF16>(p, tiles, stream);
    case kAddSkip: return launch_conv<F, kAddSkip, BF16>(p, tiles, stream);
    default: return launch_conv<F, kFsrTail, BF16>(p, tiles, stream);
    }
}

// The network over one image: head, `layers` 3x3 F->F convolutions (mode per
// layer from `plan`), upscale.  maps: three [h][w][F] 16-bit arrays.
template <typename T, int F, int K, bool BF16>
cudaError_t run_typed(const float* kernels, const float* biases, const float* alphas, bool artcnn, int blocks, const void* packed,
                      const Plane& in, const Plane& out, void* const maps[3], int* status, cudaStream_t stream)
{
    const int w = in.w, h = in.h;
    uint4* feat = static_cast<uint4*>(maps[0]);
    uint4* a = static_cast<uint4*>(maps[1]);
    uint4* bm = static_cast<uint4*>(maps[2]);
    const dim3 pgrid((w + 31) / 32, (h + 7) / 8);
    {
        HeadP<K, F> hp;
        for (int i = 0; i < F * K * K; i++) hp.k[i] = kernels[i];
        for (int i = 0; i < F; i++) hp.b[i] = biases[i];
        head_kernel<T, K, F, BF16><<<pgrid, 256, 0, stream>>>(hp, in, feat);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
        count_launch();
    }
    ConvWP<F> c;
    std::memset(&c, 0, sizeof(c));
    c.status = status;
    c.nimg = 1;
    c.img[0].w = w;
    c.img[0].h = h;
    c.img[0].tiles_x = (w + TW - 1) / TW;
    c.img[0].tile0 = 0;
    const int tiles = c.img[0].tiles_x * ((h + TH - 1) / TH);
    const size_t lb = static_cast<size_t>(9) * F * F;  // packed 16-bit values per layer
    const int hk = F * K * K;                           // head kernel floats
    const uint4* cur = feat;
    // parameters of the persistent kernel (large: thread-local, not on the stack)
    static thread_local ConvPP<F> pp_storage;
    ConvPP<F>& r = pp_storage;
    std::memset(&r, 0, sizeof(r));
    r.status = status;
    r.nimg = 1;
    r.ntiles = tiles;
    // ArtCNN: blocks ReLU layers, then identity + feat.  FSRCNNX: blocks-1
    // PReLU layers, then the tail (PReLU, 1x1 + feat, PReLU).
    const int nconv = artcnn ? blocks + 1 : blocks;
    for (int l = 1; l <= nconv; l++)
    {
        const bool last = l == nconv;
        const int mode = artcnn ? (last ? kAddSkip : kReLU) : (last ? kFsrTail : kPReLU);
        ConvWP<F> q = c;
        q.img[0].in = cur;
        q.img[0].out = a;
        q.img[0].skip = feat;
        q.bw = static_cast<const uint4*>(packed) + (l - 1) * lb * 2 / 16;
        for (int i = 0; i < F; i++)
        {
            q.b[i] = biases[F * l + i];
            q.a[i] = (!artcnn && alphas) ? alphas[F * (l - 1) + i] : 0.0f;
        }
        if (mode == kFsrTail)
        {
            for (int i = 0; i < F * F; i++) q.k1[i] = kernels[hk + F * F * 9 * blocks + i];
            for (int i = 0; i < F; i++)
            {
                q.b1[i] = biases[F * (l + 1) + i];
                q.a1[i] = alphas[F * l + i];
            }
        }
        cudaError_t err;
        if (F == 32 || mode == kFsrTail)
        {
            // 32 channels, and FSRCNNX's tail with its FP32 1x1 epilogue: the
            // persistent TMA-fed pipeline, epilogue overlapped with the MMAs
            r.bw = q.bw;
            std::memcpy(r.b, q.b, sizeof(r.b));
            std::memcpy(r.a, q.a, sizeof(r.a));
            std::memcpy(r.k1, q.k1, sizeof(r.k1));
            std::memcpy(r.b1, q.b1, sizeof(r.b1));
            std::memcpy(r.a1, q.a1, sizeof(r.a1));
            r.img[0] = ImgP{feat, a, w, h, c.img[0].tiles_x, 0, Plane{}};
            if (!encode_tmap_3d_u16(&r.tmap[0], cur, F, w, h, 8, WW, WH)) return cudaErrorInvalidValue;
            err = convp_mode<F, BF16>(mode, r, stream);
        }
        else
            // the other 16-channel layers: one CTA per tile, four per SM (measured faster here)
            err = conv_mode<F, BF16>(mode, q, tiles, stream);
        if (err != cudaSuccess) return err;
        count_launch();
        cur = a;
        uint4* t = a;
        a = bm;
        bm = t;
    }
    // upscale (ArtCNN layer blocks+2, FSRCNNX layer blocks+2 after the 1x1) on
    // the tensor core: its packed B follows the 3x3 layers'
    const int lu = blocks + 2;
    r.bw = static_cast<const uint4*>(packed) + nconv * lb * 2 / 16;
    for (int i = 0; i < 4; i++) r.b[i] = biases[F * lu + i];
    r.img[0] = ImgP{nullptr, nullptr, w, h, c.img[0].tiles_x, 0, out};
    if (!encode_tmap_3d_u16(&r.tmap[0], cur, F, w, h, 8, WW, WH)) return cudaErrorInvalidValue;
    cudaError_t err = launch_convp<F, kUp, BF16, T>(r, stream);
    if (err == cudaSuccess) count_launch();
    return err;
}

template <int F, int K, bool BF16>
cudaError_t run_type(const float* kernels, const float* biases, const float* alphas, bool artcnn, int blocks, const void* packed,
                     const Plane& in, const Plane& out, void* const maps[3], int* status, cudaStream_t stream)
{
    switch (in.type)
    {
    case kU8: return run_typed<uint8_t, F, K, BF16>(kernels, biases, alphas, artcnn, blocks, packed, in, out, maps, status, stream);
    case kU16: return run_typed<uint16_t, F, K, BF16>(kernels, biases, alphas, artcnn, blocks, packed, in, out, maps, status, stream);
    case kF32: return run_typed<float, F, K, BF16>(kernels, biases, alphas, artcnn, blocks, packed, in, out, maps, status, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace f3tc

// Packed B of the 3x3 F->F layers of an ArtCNN (blocks + 1 layers) or
// FSRCNNX (blocks layers) model, F = 16 or 32, then the upscale layer's.
void pack_f3_tc_weights(const float* kernels, int F, bool artcnn, int blocks, bool bf16, std::vector<uint16_t>& packed)
{
    const int layers = artcnn ? blocks + 1 : blocks;
    const int head = artcnn ? F * 9 : F * 25;
    const size_t lb = static_cast<size_t>(9) * F * F;
    packed.assign(layers * lb + static_cast<size_t>(9) * F * 16, 0);
    for (int l = 0; l < layers; l++) f3tc::pack_f3_conv(kernels + head + F * F * 9 * l, F, bf16, packed.data() + l * lb);
    const float* up = kernels + head + F * F * 9 * layers + (artcnn ? 0 : F * F);  // FSRCNNX: after the 1x1
    f3tc::pack_f3_up(up, F, bf16, packed.data() + layers * lb);
}

cudaError_t launch_f3_tc(const float* kernels, const float* biases, const float* alphas, bool artcnn, int F, int blocks,
                         const void* packed, bool bf16, const Plane& in, const Plane& out, void* const maps[3], int* status,
                         cudaStream_t stream)
{
    using namespace f3tc;
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    if (!packed || !status || blocks < 2 || (F != 16 && F != 32)) return cudaErrorInvalidValue;
    if (artcnn)
        return F == 32 ? (bf16 ? run_type<32, 3, true>(kernels, biases, alphas, true, blocks, packed, in, out, maps, status, stream)
                               : run_type<32, 3, false>(kernels, biases, alphas, true, blocks, packed, in, out, maps, status, stream))
                       : (bf16 ? run_type<16, 3, true>(kernels, biases, alphas, true, blocks, packed, in, out, maps, status, stream)
                               : run_type<16, 3, false>(kernels, biases, alphas, true, blocks, packed, in, out, maps, status, stream));
    if (F != 16) return cudaErrorInvalidValue;
    return bf16 ? run_type<16, 5, true>(kernels, biases, alphas, false, blocks, packed, in, out, maps, status, stream)
                : run_type<16, 5, false>(kernels, biases, alphas, false, blocks, packed, in, out, maps, status, stream);
}

}  // namespace acgb
