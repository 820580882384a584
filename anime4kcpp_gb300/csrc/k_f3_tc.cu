// ArtCNN<16/32> and FSRCNNX<16> x2 passes in a tensor-core form (FP16 or BF16
// operands, FP32 accumulation): the 3x3 F->F layers and the F->4 upscale on
// tcgen05, the 1->F head in FP32 on CUDA cores, F-channel 16-bit maps between
// launches.
//
// Networks and CPU order as k_f3_fp32.cu (CPUProcessor.cpp:1519-1600,
// 1629-1715).  Each 3x3 layer is one launch of convq_kernel: persistent CTAs
// (one per SM for F = 32, two for F = 16) walk the layer's 30 x 30 tiles (a
// 32 x 32 window, halo 1, clamped to the map's edge) with a two-stage
// pipeline (TMA window loads, one MMA lane, epilogue warps).  One GEMM row
// holds two adjacent pixels (N = 2F output columns), K = 16 channels of one
// input pixel per MMA.
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
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr int kMaxImg = 16;

enum Mode { kReLU = 0, kPReLU = 1, kAddSkip = 2, kFsrTail = 3, kUp = 4 };

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

constexpr int NSTAGE = 2;

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
    const uint4* bw;            // packed B of the layer (pack_f3_pair)
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

// ---- the persistent pair-form conv kernel ----
// Persistent CTAs walk a layer's tiles with a two-stage pipeline: while the
// epilogue warps drain tile t's accumulators, the MMA lane runs tile t + 1
// and the producer warp loads tile t + 2's window with TMA (the out-of-image
// ring that clamp-to-edge needs is then copied in from its neighbours).
// Stage s of tile t (s = t % 2, u = t / 2):
//   full[s]   TMA bytes of the window landed          (producer waits)
//   ready[s]  window complete, edge ring filled       (MMA lane waits)
//   mdone[s]  MMAs of the stage completed (commit)    (epilogue, producer wait)
//   tfree[s]  accumulators drained by every epilogue warp (MMA lane waits)
// Each wait targets completion u (or u - 1) of a barrier whose next completion
// needs the waiter's own progress, so no phase is ever skipped.  Every wait is
// bounded; a timeout raises the CTA's abort flag and the status word.
//
// One GEMM row holds two horizontally adjacent pixels (N = 2F), which reads
// the A operand from shared memory a fifth (F = 32) to a quarter (F = 16)
// less often per output pixel than one pixel per row.  The window is held as
// [parity][8-channel group] planes of 16-byte pair slots (TMA loads each with
// a traversal stride of 2 pixels).  For tap row dy and input pixel offset o
// in {-1, 0, 1, 2} from the pair's first pixel, the K16 chunk of channels
// 16 j .. 16 j + 15 is a shifted view of the parity-(o & 1) planes of groups
// 2 j and 2 j + 1 (leading byte offset one plane) at pair shift floor(o / 2);
// output pixel k takes that input through tap dx = o - k + 1 (zero weight
// outside 0..2).  12 F/16 MMAs per 128 pairs.
//
// Modes: the 3x3 F -> F layer with ReLU, PReLU, + feat (ArtCNN's last), or
// FSRCNNX's tail (PReLU, conv1x1 F -> F, + feat, PReLU) in the epilogue; kUp:
// the F -> 4 upscale with N = 32 (per output pixel: the weights' 16-bit high
// parts in columns 0-3, their residuals in 4-7), pixel-shuffled into the OT
// plane.
constexpr int PPR = WW / 2;                     // pairs per window row
constexpr int NB2 = WW * WH / 2 / 128;          // 4 blocks of 128 pair rows
constexpr int PAD2 = 24;                        // >= PPR + 1; PAD2 * 16 a multiple of 128 (TMA)
constexpr int PLANE2 = (PAD2 + NB2 * 128 + PAD2) * 16;

template <int F>
struct GeoQ
{
    static constexpr int NG = F / 8;                 // channel groups
    static constexpr int NPL = 2 * NG;               // planes [parity][group]
    static constexpr int WIN_BYTES = NPL * PLANE2;
    static constexpr int N = 2 * F;                  // MMA N of the 3x3 F -> F layers
    static constexpr int B_BYTES = 12 * (F / 16) * N * 32;
    static constexpr uint32_t TMEM_COLS = NSTAGE * NB2 * N;  // 256 (F = 16) or 512 (F = 32)
    static constexpr int NEPI = F == 32 ? 16 : 8;
    static constexpr int THREADS = (2 + NEPI) * 32;
    static constexpr int MINB = F == 32 ? 1 : 2;
    static constexpr int BAR_OFF = NSTAGE * WIN_BYTES + B_BYTES;
    static constexpr int SMEM = BAR_OFF + 128;
    static constexpr int MIN_SMEM = (228 * 1024) / (512 / TMEM_COLS + 1) + 1024;
    static constexpr int SMEM_REQ = SMEM > MIN_SMEM ? SMEM : MIN_SMEM;
    static constexpr uint32_t BOX_BYTES = 8 * PPR * WH * 2;  // one parity-group plane
    static_assert((PAD2 * 16) % 128 == 0 && PLANE2 % 128 == 0, "TMA destinations 128-byte aligned");
    static_assert(PAD2 >= PPR + 1, "taps of the first and last rows stay inside a plane");
};

template <int F, int MODE, bool BF16, typename OT>
__global__ void __launch_bounds__(GeoQ<F>::THREADS, GeoQ<F>::MINB) convq_kernel(const __grid_constant__ ConvPP<F> P)
{
    using G = GeoQ<F>;
    constexpr int NG = G::NG, NEPI = G::NEPI;
    constexpr int NM = MODE == kUp ? 32 : G::N;  // MMA N
    constexpr int CHUNK_M = NM * 32;
    constexpr int BB = 12 * (F / 16) * CHUNK_M;
    static_assert(BB <= G::B_BYTES, "B fits its buffer");
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* bsm = smem + NSTAGE * G::WIN_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + G::BAR_OFF);
    uint64_t* full = bars;
    uint64_t* ready = bars + 2;
    uint64_t* mdone = bars + 4;
    uint64_t* tfree = bars + 6;
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
    for (int i = tid; i < NSTAGE * G::NPL * 2 * PAD2; i += G::THREADS)
    {
        const int pl = i / (2 * PAD2), k = i % (2 * PAD2);
        reinterpret_cast<uint4*>(smem + pl * PLANE2)[k < PAD2 ? k : NB2 * 128 + k] = make_uint4(0, 0, 0, 0);
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
        bool pending = false;
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
                tc::mbar_arrive_expect_tx(&full[s], G::NPL * G::BOX_BYTES);
#pragma unroll
                for (int e = 0; e < 2; e++)
#pragma unroll
                    for (int g = 0; g < NG; g++)
                        tc::tma_load_3d(win + (e * NG + g) * PLANE2 + PAD2 * 16, &P.tmap[im], 8 * g, x0 + e, y0, &full[s]);
            }
            pending = true;
            ok = wait_bar(&full[s], u & 1u, abort_flag);
            if (!__all_sync(0xffffffffu, ok ? 1 : 0)) break;
            pending = false;
            // clamp-to-edge ring: window column wx lives in parity plane wx & 1 at pair wx >> 1
            const int xl = x0 < 0 ? 0 : -1, xr = I.w - x0 < WW ? I.w - x0 : -1;
            const int yt = y0 < 0 ? 0 : -1, yb = I.h - y0 < WH ? I.h - y0 : -1;
            if (xl >= 0 || xr >= 0 || yt >= 0 || yb >= 0)
            {
                uint4* pw = reinterpret_cast<uint4*>(win) + PAD2;
                auto at = [&](int wx, int wy, int g) -> uint4& {
                    return pw[((wx & 1) * NG + g) * (PLANE2 / 16) + wy * PPR + (wx >> 1)];
                };
                for (int i = lane; i < WH * NG; i += 32)
                {
                    const int wy = i / NG, g = i % NG;
                    if (xl >= 0) at(xl, wy, g) = at(xl + 1, wy, g);
                    if (xr >= 0) at(xr, wy, g) = at(xr - 1, wy, g);
                }
                __syncwarp();
                for (int i = lane; i < WW * NG; i += 32)
                {
                    const int wx = i / NG, g = i % NG;
                    if (yt >= 0) at(wx, yt, g) = at(wx, yt + 1, g);
                    if (yb >= 0) at(wx, yb, g) = at(wx, yb - 1, g);
                }
                tc::fence_proxy_async_smem();
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&ready[s]);
        }
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
            const uint64_t bdesc = tc::smem_desc(tc::smem_u32(bsm), NM * 16, 128);
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
                const uint64_t adesc = tc::smem_desc(tc::smem_u32(smem + s * G::WIN_BYTES), PLANE2, 128);
#pragma unroll 1
                for (int b = 0; b < NB2; b++)
                {
                    const uint32_t d = tmem + static_cast<uint32_t>((s * NB2 + b) * G::N);
                    const uint64_t ab = adesc + static_cast<uint64_t>(PAD2 + 128 * b);
#pragma unroll
                    for (int dy = 0; dy < 3; dy++)
#pragma unroll
                        for (int oi = 0; oi < 4; oi++)
#pragma unroll
                            for (int j2 = 0; j2 < F / 16; j2++)
                            {
                                // input offset o = oi - 1: parity o & 1, pair shift floor(o / 2)
                                constexpr int PL16 = PLANE2 / 16;
                                const int par = (oi + 1) & 1, dp = (oi == 0) ? -1 : (oi == 3 ? 1 : 0);
                                const int off = (par * NG + 2 * j2) * PL16 + (dy - 1) * PPR + dp;
                                const int ch = (dy * 4 + oi) * (F / 16) + j2;
                                tc::mma_f16(d, ab + static_cast<uint64_t>(static_cast<int64_t>(off)),
                                            bdesc + static_cast<uint64_t>(ch * (CHUNK_M / 16)), IDESC, (dy | oi | j2) ? 1u : 0u);
                            }
                }
                tc::mma_commit(&mdone[s]);
                last = it;
            }
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
            for (int b = part; b < NB2; b += NEPI / 4)
            {
                const int r = b * 128 + q4 * 32 + lane;  // this lane's pair row
                const int y = r / PPR, xp = 2 * (r - y * PPR);
                const uint32_t tl = tmem + (static_cast<uint32_t>(q4 * 32) << 16) + static_cast<uint32_t>((s * NB2 + b) * G::N);
#pragma unroll
                for (int kp = 0; kp < 2; kp++)
                {
                    const int x = xp + kp, gx = x0 + x, gy = y0 + y;
                    const bool valid = !(y < 1 || y > TH || x < 1 || x > TW || gx >= I.w || gy >= I.h);
                    if constexpr (MODE == kUp)
                    {
                        float q[16];
                        tc::tmem_ld16(tl + static_cast<uint32_t>(16 * kp), q);
                        tc::tmem_wait_ld();
                        if (!valid) continue;
                        OT* r0 = row_ptr_w<OT>(I.dst.ptr, I.dst.pitch, 2 * gy) + 2 * gx;
                        OT* r1 = row_ptr_w<OT>(I.dst.ptr, I.dst.pitch, 2 * gy + 1) + 2 * gx;
                        r0[0] = from_float<OT>(q[0] + q[4] + P.b[0]);
                        r0[1] = from_float<OT>(q[1] + q[5] + P.b[1]);
                        r1[0] = from_float<OT>(q[2] + q[6] + P.b[2]);
                        r1[1] = from_float<OT>(q[3] + q[7] + P.b[3]);
                        continue;
                    }
                    else
                    {
                        float v[F];
#pragma unroll
                        for (int h = 0; h < F / 16; h++)
                        {
                            float q[16];
                            tc::tmem_ld16(tl + static_cast<uint32_t>(kp * F + 16 * h), q);
                            tc::tmem_wait_ld();
#pragma unroll
                            for (int c = 0; c < 16; c++) v[16 * h + c] = q[c];
                        }
                        if (!valid) continue;
                        const size_t o = (static_cast<size_t>(gy) * I.w + gx) * NG;
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
                            for (int j = 0; j < NG; j++)
                            {
                                float sk[8];
                                unpack8<BF16>(I.skip[o + j], sk);
#pragma unroll
                                for (int c = 0; c < 8; c++) v[8 * j + c] += sk[c];
                            }
                        }
                        if constexpr (MODE == kFsrTail)
                        {
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
                            for (int j = 0; j < NG; j++)
                            {
                                float f[8];
                                unpack8<BF16>(I.skip[o + j], f);
#pragma unroll
                                for (int c = 0; c < 8; c++) v[8 * j + c] = prelu(uo[8 * j + c] + f[c], P.a1[8 * j + c]);
                            }
                        }
#pragma unroll
                        for (int j = 0; j < NG; j++) I.out[o + j] = pack8<BF16>(v + 8 * j);
                    }
                }
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
    Plane in[kMaxImg];  // image blockIdx.z
    uint4* feat[kMaxImg];
};

// conv KxK 1 -> F (identity) in FP32 from the input plane, taps clamped,
// stored as an F-channel 16-bit map; blockIdx.z picks the image.
template <typename T, int K, int F, bool BF16>
__global__ void __launch_bounds__(256) head_kernel(const __grid_constant__ HeadP<K, F> W)
{
    constexpr int R = K / 2, SW = 32 + 2 * R, SH = 8 + 2 * R;
    const Plane& in = W.in[blockIdx.z];
    uint4* __restrict__ feat = W.feat[blockIdx.z];
    // the block's 32 x 8 pixels with their clamped halo, converted once
    __shared__ float s[SH][SW];
    const int bx = blockIdx.x * 32, by = blockIdx.y * 8;
    if (bx >= in.w || by >= in.h) return;  // the grid covers the largest image of the launch
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

// The pair form of one 3x3 F->F layer k[n * 9F + tap * F + c] (up = false,
// N = 2F) or of the F->4 upscale (up = true, N = 32: per output pixel the
// 16-bit weights of outputs 0..3, their residuals, eight zero columns): chunk
// (dy, oi, j2) at (dy * 4 + oi) F/16 + j2, input pixel offset o = oi - 1,
// channels 16 j2 .. 16 j2 + 15; column n is output pixel n / (N / 2), channel
// n % (N / 2), fed through tap dx = o - n / (N / 2) + 1.  Element (n, kk) at
// byte (kk / 8) 16 N + (n / 8) 128 + (n % 8) 16 + (kk % 8) 2.
void pack_f3_pair(const float* k, int F, bool up, bool bf16, uint16_t* out)
{
    const int N = up ? 32 : 2 * F, half = N / 2;
    const size_t chunk = static_cast<size_t>(N) * 16;  // 16-bit values
    std::memset(out, 0, 12 * (F / 16) * chunk * 2);
    for (int dy = 0; dy < 3; dy++)
        for (int oi = 0; oi < 4; oi++)
            for (int j2 = 0; j2 < F / 16; j2++)
            {
                uint16_t* ch = out + ((dy * 4 + oi) * (F / 16) + j2) * chunk;
                for (int n = 0; n < N; n++)
                {
                    const int kp = n / half, m = n % half, dx = (oi - 1) - kp + 1;
                    if (dx < 0 || dx > 2 || (up && m >= 8)) continue;
                    for (int kk = 0; kk < 16; kk++)
                    {
                        const int c = 16 * j2 + kk;
                        const float wv = k[(up ? (m & 3) : m) * 9 * F + (dy * 3 + dx) * F + c];
                        uint16_t bits = to_bits(wv, bf16);
                        if (up && m >= 4) bits = to_bits(wv - from_bits(to_bits(wv, bf16), bf16), bf16);
                        ch[((kk >> 3) * 16 * N + (n >> 3) * 128 + (n & 7) * 16 + (kk & 7) * 2) / 2] = bits;
                    }
                }
            }
}

template <int F, int MODE, bool BF16, typename OT = uint8_t>
cudaError_t launch_convq(const ConvPP<F>& p, cudaStream_t stream)
{
    using G = GeoQ<F>;
    // one-time set-up per device, thread-safe
    const LaunchSetup setup = device_once([] {
        cudaError_t err =
            cudaFuncSetAttribute(convq_kernel<F, MODE, BF16, OT>, cudaFuncAttributeMaxDynamicSharedMemorySize, G::SMEM_REQ);
        if (err != cudaSuccess) return LaunchSetup{err, 0, 0};
        int occ = 0, dev = 0, sms = 0;
        if ((err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, convq_kernel<F, MODE, BF16, OT>, G::THREADS, G::SMEM_REQ)) !=
            cudaSuccess)
            return LaunchSetup{err, 0, 0};
        if ((err = cudaGetDevice(&dev)) != cudaSuccess) return LaunchSetup{err, 0, 0};
        if ((err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return LaunchSetup{err, 0, 0};
        if (occ < 1) return LaunchSetup{cudaErrorInvalidConfiguration, 0, 0};
        const int cap = static_cast<int>(512 / G::TMEM_COLS);
        return LaunchSetup{cudaSuccess, occ < cap ? occ : cap, sms};
    });
    if (setup.err != cudaSuccess) return setup.err;
    const int per_sm = setup.per_sm, sms = setup.sms;
    const int grid = p.ntiles < per_sm * sms ? p.ntiles : per_sm * sms;
    convq_kernel<F, MODE, BF16, OT><<<grid, G::THREADS, G::SMEM_REQ, stream>>>(p);
    return cudaGetLastError();
}

template <int F, bool BF16>
cudaError_t convq_mode(int mode, const ConvPP<F>& p, cudaStream_t stream)
{
    switch (mode)
    {
    case kReLU: return launch_convq<F, kReLU, BF16>(p, stream);
    case kPReLU: return launch_convq<F, kPReLU, BF16>(p, stream);
    case kAddSkip: return launch_convq<F, kAddSkip, BF16>(p, stream);
    default: return launch_convq<F, kFsrTail, BF16>(p, stream);
    }
}

// One head launch over n images (grid z = image).
template <typename T, int K, int F, bool BF16>
cudaError_t launch_head(const float* kernels, const float* biases, int n, const Plane* in, uint4* const* feat, cudaStream_t stream)
{
    HeadP<K, F> hp;
    for (int i = 0; i < F * K * K; i++) hp.k[i] = kernels[i];
    for (int i = 0; i < F; i++) hp.b[i] = biases[i];
    int mw = 0, mh = 0;
    for (int i = 0; i < n; i++)
    {
        hp.in[i] = in[i];
        hp.feat[i] = feat[i];
        mw = in[i].w > mw ? in[i].w : mw;
        mh = in[i].h > mh ? in[i].h : mh;
    }
    head_kernel<T, K, F, BF16><<<dim3((mw + 31) / 32, (mh + 7) / 8, n), 256, 0, stream>>>(hp);
    return cudaGetLastError();
}

// The network over n images (one launch per layer over all of them): head,
// the 3x3 F->F layers (ArtCNN: blocks ReLU layers, then identity + feat;
// FSRCNNX: blocks - 1 PReLU layers, then the tail: PReLU, 1x1 + feat,
// PReLU), upscale.  maps[3 i + j]: image i's three [h][w][F] 16-bit arrays;
// packed: pack_f3_tc_weights().
template <typename T, int F, int K, bool BF16>
cudaError_t run_typed(const float* kernels, const float* biases, const float* alphas, bool artcnn, int blocks, const void* packed,
                      int n, const Plane* in, const Plane* out, void* const* maps, int* status, cudaStream_t stream)
{
    uint4* feat[kMaxImg];
    for (int i = 0; i < n; i++) feat[i] = static_cast<uint4*>(maps[3 * i]);
    cudaError_t err = launch_head<T, K, F, BF16>(kernels, biases, n, in, feat, stream);
    if (err != cudaSuccess) return err;
    count_launch();
    // kernel parameters (large: thread-local, not on the stack)
    static thread_local ConvPP<F> pp_storage;
    ConvPP<F>& r = pp_storage;
    std::memset(&r, 0, sizeof(r));
    r.status = status;
    r.nimg = n;
    int tiles_x[kMaxImg], tile0[kMaxImg];
    r.ntiles = 0;
    for (int i = 0; i < n; i++)
    {
        tiles_x[i] = (in[i].w + TW - 1) / TW;
        tile0[i] = r.ntiles;
        r.ntiles += tiles_x[i] * ((in[i].h + TH - 1) / TH);
    }
    const size_t lb = static_cast<size_t>(24) * F * F;  // packed 16-bit values per 3x3 layer
    const int hk = F * K * K;                           // head kernel floats
    int cur = 0, a = 1, bm = 2;                         // map slots: input, output, spare
    const int nconv = artcnn ? blocks + 1 : blocks;
    for (int l = 1; l <= nconv; l++)
    {
        const bool last = l == nconv;
        const int mode = artcnn ? (last ? kAddSkip : kReLU) : (last ? kFsrTail : kPReLU);
        r.bw = static_cast<const uint4*>(packed) + (l - 1) * lb * 2 / 16;
        for (int i = 0; i < F; i++)
        {
            r.b[i] = biases[F * l + i];
            r.a[i] = (!artcnn && alphas) ? alphas[F * (l - 1) + i] : 0.0f;
        }
        if (mode == kFsrTail)
        {
            for (int i = 0; i < F * F; i++) r.k1[i] = kernels[hk + F * F * 9 * blocks + i];
            for (int i = 0; i < F; i++)
            {
                r.b1[i] = biases[F * (l + 1) + i];
                r.a1[i] = alphas[F * l + i];
            }
        }
        for (int i = 0; i < n; i++)
        {
            r.img[i] = ImgP{feat[i], static_cast<uint4*>(maps[3 * i + a]), in[i].w, in[i].h, tiles_x[i], tile0[i], Plane{}};
            if (!encode_tmap_3d_u16_strided(&r.tmap[i], maps[3 * i + cur], F, in[i].w, in[i].h, 8, WW, WH, 2))
                return cudaErrorInvalidValue;
        }
        if ((err = convq_mode<F, BF16>(mode, r, stream)) != cudaSuccess) return err;
        count_launch();
        cur = a;  // this layer's output feeds the next; output and spare swap
        const int t = a;
        a = bm;
        bm = t;
    }
    // upscale (layer blocks + 2 of both families; FSRCNNX's after the 1x1)
    const int lu = blocks + 2;
    r.bw = static_cast<const uint4*>(packed) + nconv * lb * 2 / 16;
    for (int i = 0; i < 4; i++) r.b[i] = biases[F * lu + i];
    for (int i = 0; i < n; i++)
    {
        r.img[i] = ImgP{nullptr, nullptr, in[i].w, in[i].h, tiles_x[i], tile0[i], out[i]};
        if (!encode_tmap_3d_u16_strided(&r.tmap[i], maps[3 * i + cur], F, in[i].w, in[i].h, 8, WW, WH, 2))
            return cudaErrorInvalidValue;
    }
    err = launch_convq<F, kUp, BF16, T>(r, stream);
    if (err == cudaSuccess) count_launch();
    return err;
}

template <int F, int K, bool BF16>
cudaError_t run_type(const float* kernels, const float* biases, const float* alphas, bool artcnn, int blocks, const void* packed,
                     int n, const Plane* in, const Plane* out, void* const* maps, int* status, cudaStream_t stream)
{
    switch (in[0].type)
    {
    case kU8:
        return run_typed<uint8_t, F, K, BF16>(kernels, biases, alphas, artcnn, blocks, packed, n, in, out, maps, status, stream);
    case kU16:
        return run_typed<uint16_t, F, K, BF16>(kernels, biases, alphas, artcnn, blocks, packed, n, in, out, maps, status, stream);
    case kF32:
        return run_typed<float, F, K, BF16>(kernels, biases, alphas, artcnn, blocks, packed, n, in, out, maps, status, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace f3tc

// Packed B of the 3x3 F->F layers of an ArtCNN (blocks + 1 layers) or
// FSRCNNX (blocks layers) model, F = 16 or 32 (24 F F 16-bit values each),
// then the upscale layer's (12 F/16 x 512).
void pack_f3_tc_weights(const float* kernels, int F, bool artcnn, int blocks, bool bf16, std::vector<uint16_t>& packed)
{
    const int layers = artcnn ? blocks + 1 : blocks;
    const int head = artcnn ? F * 9 : F * 25;
    const float* up = kernels + head + F * F * 9 * layers + (artcnn ? 0 : F * F);  // FSRCNNX: after the 1x1
    const size_t lb = static_cast<size_t>(24) * F * F;
    packed.assign(layers * lb + static_cast<size_t>(12) * (F / 16) * 32 * 16, 0);
    for (int l = 0; l < layers; l++) f3tc::pack_f3_pair(kernels + head + F * F * 9 * l, F, false, bf16, packed.data() + l * lb);
    f3tc::pack_f3_pair(up, F, true, bf16, packed.data() + layers * lb);
}

// FSRCNNX<8>'s conv5x5 1->8 head (identity) in FP32 into 8-channel 16-bit
// maps [h][w] x 16 bytes, one launch over n images of one element type.
cudaError_t launch_f3_head8(const float* kernels, const float* biases, bool bf16, int n, const Plane* in, void* const* feat,
                            cudaStream_t stream)
{
    using namespace f3tc;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxImg) return cudaErrorInvalidValue;
    uint4* f[kMaxImg];
    for (int i = 0; i < n; i++)
    {
        if (in[i].w <= 0 || in[i].h <= 0 || in[i].type != in[0].type) return cudaErrorInvalidValue;
        f[i] = static_cast<uint4*>(feat[i]);
    }
    switch (in[0].type)
    {
    case kU8:
        return bf16 ? launch_head<uint8_t, 5, 8, true>(kernels, biases, n, in, f, stream)
                    : launch_head<uint8_t, 5, 8, false>(kernels, biases, n, in, f, stream);
    case kU16:
        return bf16 ? launch_head<uint16_t, 5, 8, true>(kernels, biases, n, in, f, stream)
                    : launch_head<uint16_t, 5, 8, false>(kernels, biases, n, in, f, stream);
    case kF32:
        return bf16 ? launch_head<float, 5, 8, true>(kernels, biases, n, in, f, stream)
                    : launch_head<float, 5, 8, false>(kernels, biases, n, in, f, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_f3_tc_batch(const float* kernels, const float* biases, const float* alphas, bool artcnn, int F, int blocks,
                               const void* packed, bool bf16, int n, const Plane* in, const Plane* out, void* const* maps,
                               int* status, cudaStream_t stream)
{
    using namespace f3tc;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxImg || !packed || !status || !maps || blocks < 2 || (F != 16 && F != 32) || (!artcnn && F != 16))
        return cudaErrorInvalidValue;
    for (int i = 0; i < n; i++)
        if (in[i].w <= 0 || in[i].h <= 0 || in[i].type != in[0].type || in[i].channels != 1 || out[i].channels != 1 ||
            out[i].w != 2 * in[i].w || out[i].h != 2 * in[i].h)
            return cudaErrorInvalidValue;
    if (artcnn)
        return F == 32 ? (bf16 ? run_type<32, 3, true>(kernels, biases, alphas, true, blocks, packed, n, in, out, maps, status, stream)
                               : run_type<32, 3, false>(kernels, biases, alphas, true, blocks, packed, n, in, out, maps, status, stream))
                       : (bf16 ? run_type<16, 3, true>(kernels, biases, alphas, true, blocks, packed, n, in, out, maps, status, stream)
                               : run_type<16, 3, false>(kernels, biases, alphas, true, blocks, packed, n, in, out, maps, status, stream));
    return bf16 ? run_type<16, 5, true>(kernels, biases, alphas, false, blocks, packed, n, in, out, maps, status, stream)
                : run_type<16, 5, false>(kernels, biases, alphas, false, blocks, packed, n, in, out, maps, status, stream);
}

cudaError_t launch_f3_tc(const float* kernels, const float* biases, const float* alphas, bool artcnn, int F, int blocks,
                         const void* packed, bool bf16, const Plane& in, const Plane& out, void* const maps[3], int* status,
                         cudaStream_t stream)
{
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    return launch_f3_tc_batch(kernels, biases, alphas, artcnn, F, blocks, packed, bf16, 1, &in, &out, maps, status, stream);
}

}  // namespace acgb
