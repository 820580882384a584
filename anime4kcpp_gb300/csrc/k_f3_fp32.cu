// ArtCNN<16/32> and FSRCNNX<8/16> x2 passes in plain FP32, one kernel per
// layer (up to two for 32-channel layers).
//
// Networks (core/src/processor/cpu/CPUProcessor.cpp:1519-1600, 1629-1715;
// layer templates core/internal/AC/Core/Internal/Processor/CPU/Common.hpp):
//   ArtCNN<F>   conv3x3 1->F identity -> feat; blocks x conv3x3 F->F + ReLU;
//               conv3x3 F->F identity + feat; conv3x3 F->4, pixel shuffle
//   FSRCNNX<F>  conv5x5 1->F identity -> feat; blocks-1 x conv3x3 F->F +
//               PReLU; conv3x3 F->F + PReLU, conv1x1 F->F + feat, PReLU;
//               conv3x3 F->4, pixel shuffle
// All taps clamp to the map's edge.  The F-channel FP32 maps live in HBM
// ([h][w][F]); a block of 256 threads computes a 32x8 pixel tile from its
// haloed input tile staged in shared memory, one pixel per thread.  A layer's
// weights travel as a by-value kernel parameter (a 32-channel layer runs as
// two launches of 16 output channels each, so they stay within the parameter
// limit); layers of more than 1,024 weights (the 16/32-channel ones) copy
// them into shared memory per block, where the inner loop reads four channels
// at a time as warp-wide broadcasts, the 8-channel ones use them straight from
// the constant bank (they fit its cache).
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.hpp"

namespace acgb {
namespace f3 {

constexpr int BX = 32, BY = 8, THREADS = BX * BY;
constexpr int SX = BX + 2, SY = BY + 2;

enum Act { kIdentity = 0, kReLU = 1, kPReLU = 2 };

__device__ __forceinline__ float act(float v, int kind, float a)
{
    if (kind == kReLU) return fmaxf(v, 0.0f);
    if (kind == kPReLU) return fmaxf(v, 0.0f) + a * fminf(v, 0.0f);
    return v;
}

template <int K, int F>
struct HeadW
{
    float k[F * K * K];
    float b[F];
};

// conv KxK 1 -> F (identity) from the input plane, taps clamped.
template <typename T, int K, int F>
__global__ void __launch_bounds__(THREADS) head_kernel(const __grid_constant__ HeadW<K, F> W, Plane in, float* __restrict__ feat)
{
    constexpr int R = K / 2;
    __shared__ float s[BY + 2 * R][BX + 2 * R];
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    for (int i = threadIdx.x; i < (BX + 2 * R) * (BY + 2 * R); i += THREADS)
    {
        const int sy = i / (BX + 2 * R), sx = i % (BX + 2 * R);
        const int gx = clampi(x0 - R + sx, 0, in.w - 1), gy = clampi(y0 - R + sy, 0, in.h - 1);
        s[sy][sx] = to_float<T>(row_ptr<T>(in.ptr, in.pitch, gy)[gx]);
    }
    __syncthreads();
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= in.w || y >= in.h) return;
    float* o = feat + (static_cast<size_t>(y) * in.w + x) * F;
#pragma unroll
    for (int n0 = 0; n0 < F; n0 += 4)
    {
        float r[4];
#pragma unroll
        for (int j = 0; j < 4; j++)
        {
            float v = W.b[n0 + j];
#pragma unroll
            for (int p = 0; p < K * K; p++) v = fmaf(s[ty + p / K][tx + p % K], W.k[(n0 + j) * K * K + p], v);
            r[j] = v;
        }
        reinterpret_cast<float4*>(o)[n0 / 4] = make_float4(r[0], r[1], r[2], r[3]);
    }
}

template <int CIN, int NB>
struct ConvW
{
    float k[NB * 9 * CIN];  // output channels n0 .. n0+NB-1: k[(n - n0) * 9 * CIN + tap * CIN + c]
    float b[NB];
    float a[NB];            // PReLU slopes
};

// Whether a layer's weights go to shared memory (more than 1,024 floats).
template <int CIN, int NB>
constexpr bool kSmemWeights = NB * 9 * CIN > 1024;

// Stage the haloed tile (SX x SY pixels of CIN floats, clamped) into smem.
template <int CIN>
__device__ __forceinline__ void stage(float4* s, const float* in, int w, int h, int x0, int y0)
{
    constexpr int V = CIN / 4;
    for (int i = threadIdx.x; i < SX * SY * V; i += THREADS)
    {
        const int v = i % V, px = i / V;
        const int sy = px / SX, sx = px % SX;
        const int gx = clampi(x0 - 1 + sx, 0, w - 1), gy = clampi(y0 - 1 + sy, 0, h - 1);
        s[i] = reinterpret_cast<const float4*>(in + (static_cast<size_t>(gy) * w + gx) * CIN)[v];
    }
}

// conv3x3 CIN -> output channels n0 .. n0+NB-1 (of COUT in the output map) +
// activation, optionally + skip (scale 1).
template <int CIN, int NB, int ACT, bool RES>
__global__ void __launch_bounds__(THREADS) conv_kernel(const __grid_constant__ ConvW<CIN, NB> W, const float* __restrict__ in,
                                                       float* __restrict__ out, const float* __restrict__ skip, int cout, int n0,
                                                       int w, int h)
{
    extern __shared__ float4 s4[];
    constexpr int V = CIN / 4;
    float4* wsm = s4 + SX * SY * V;  // weights: [n][tap][CIN / 4]
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    stage<CIN>(s4, in, w, h, x0, y0);
    if constexpr (kSmemWeights<CIN, NB>)
        for (int i = threadIdx.x; i < NB * 9 * V; i += THREADS)
            wsm[i] = make_float4(W.k[4 * i], W.k[4 * i + 1], W.k[4 * i + 2], W.k[4 * i + 3]);
    __syncthreads();
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= w || y >= h) return;
    float acc[NB];
#pragma unroll
    for (int n = 0; n < NB; n++) acc[n] = W.b[n];
    if constexpr (!kSmemWeights<CIN, NB>)
    {
        // weights straight from the constant bank
#pragma unroll
        for (int p = 0; p < 9; p++)
        {
            const float4* px = s4 + ((ty + p / 3) * SX + tx + p % 3) * V;
#pragma unroll
            for (int v = 0; v < V; v++)
            {
                const float4 u = px[v];
                const float xv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int n = 0; n < NB; n++) acc[n] = fmaf(xv[j], W.k[n * 9 * CIN + p * CIN + 4 * v + j], acc[n]);
            }
        }
    }
    else
    {
#pragma unroll 1
        for (int p = 0; p < 9; p++)
        {
            const float4* px = s4 + ((ty + p / 3) * SX + tx + p % 3) * V;
            const float4* wp = wsm + p * V;
#pragma unroll 2
            for (int v = 0; v < V; v++)
            {
                const float4 u = px[v];
#pragma unroll
                for (int n = 0; n < NB; n++)
                {
                    const float4 k4 = wp[n * 9 * V + v];
                    acc[n] = fmaf(u.x, k4.x, acc[n]);
                    acc[n] = fmaf(u.y, k4.y, acc[n]);
                    acc[n] = fmaf(u.z, k4.z, acc[n]);
                    acc[n] = fmaf(u.w, k4.w, acc[n]);
                }
            }
        }
    }
    const size_t o = (static_cast<size_t>(y) * w + x) * cout + n0;
#pragma unroll
    for (int n = 0; n < NB; n += 4)
    {
        float r[4];
#pragma unroll
        for (int j = 0; j < 4; j++)
        {
            float v = act(acc[n + j], ACT, W.a[n + j]);
            if (RES) v += skip[o + n + j];
            r[j] = v;
        }
        reinterpret_cast<float4*>(out + o)[n / 4] = make_float4(r[0], r[1], r[2], r[3]);
    }
}

template <int F>
struct TailW
{
    ConvW<F, F> c3;  // conv3x3 + PReLU
    float k1[F * F];  // conv1x1 k1[n * F + c]
    float b1[F];
    float a1[F];
};

// FSRCNNX tail: conv3x3 F->F + PReLU, conv1x1 F->F + bias, + feat, PReLU.
template <int F>
__global__ void __launch_bounds__(THREADS) tail_kernel(const __grid_constant__ TailW<F> W, const float* __restrict__ in,
                                                       const float* __restrict__ feat, float* __restrict__ out, int w, int h)
{
    extern __shared__ float4 s4[];
    constexpr int V = F / 4;
    float4* wsm = s4 + SX * SY * V;  // 3x3 weights: [n][tap][F / 4]
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    stage<F>(s4, in, w, h, x0, y0);
    if constexpr (kSmemWeights<F, F>)
        for (int i = threadIdx.x; i < F * 9 * V; i += THREADS)
            wsm[i] = make_float4(W.c3.k[4 * i], W.c3.k[4 * i + 1], W.c3.k[4 * i + 2], W.c3.k[4 * i + 3]);
    __syncthreads();
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= w || y >= h) return;
    float acc[F];
#pragma unroll
    for (int n = 0; n < F; n++) acc[n] = W.c3.b[n];
    if constexpr (!kSmemWeights<F, F>)
    {
#pragma unroll
        for (int p = 0; p < 9; p++)
        {
            const float4* px = s4 + ((ty + p / 3) * SX + tx + p % 3) * V;
#pragma unroll
            for (int v = 0; v < V; v++)
            {
                const float4 u = px[v];
                const float xv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int n = 0; n < F; n++) acc[n] = fmaf(xv[j], W.c3.k[n * 9 * F + p * F + 4 * v + j], acc[n]);
            }
        }
    }
    else
    {
#pragma unroll 1
        for (int p = 0; p < 9; p++)
        {
            const float4* px = s4 + ((ty + p / 3) * SX + tx + p % 3) * V;
            const float4* wp = wsm + p * V;
#pragma unroll 2
            for (int v = 0; v < V; v++)
            {
                const float4 u = px[v];
#pragma unroll
                for (int n = 0; n < F; n++)
                {
                    const float4 k4 = wp[n * 9 * V + v];
                    acc[n] = fmaf(u.x, k4.x, acc[n]);
                    acc[n] = fmaf(u.y, k4.y, acc[n]);
                    acc[n] = fmaf(u.z, k4.z, acc[n]);
                    acc[n] = fmaf(u.w, k4.w, acc[n]);
                }
            }
        }
    }
#pragma unroll
    for (int n = 0; n < F; n++) acc[n] = act(acc[n], kPReLU, W.c3.a[n]);
    const size_t o = (static_cast<size_t>(y) * w + x) * F;
#pragma unroll
    for (int n = 0; n < F; n += 4)
    {
        float r[4];
#pragma unroll
        for (int j = 0; j < 4; j++)
        {
            float v = W.b1[n + j];
#pragma unroll
            for (int c = 0; c < F; c++) v = fmaf(acc[c], W.k1[(n + j) * F + c], v);
            r[j] = act(v + feat[o + n + j], kPReLU, W.a1[n + j]);
        }
        reinterpret_cast<float4*>(out + o)[n / 4] = make_float4(r[0], r[1], r[2], r[3]);
    }
}

template <int F>
struct UpW
{
    float k[4 * 9 * F];
    float b[4];
};

// conv3x3 F->4 (identity), pixel shuffle 2x2, fromFloat; no nearest add.
template <typename T, int F>
__global__ void __launch_bounds__(THREADS) up_kernel(const __grid_constant__ UpW<F> W, const float* __restrict__ in, Plane dst,
                                                     int w, int h)
{
    extern __shared__ float4 s4[];
    constexpr int V = F / 4;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    stage<F>(s4, in, w, h, x0, y0);
    __syncthreads();
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= w || y >= h) return;
    float acc[4];
#pragma unroll
    for (int n = 0; n < 4; n++) acc[n] = W.b[n];
#pragma unroll
    for (int p = 0; p < 9; p++)
    {
        const float4* px = s4 + ((ty + p / 3) * SX + tx + p % 3) * V;
#pragma unroll
        for (int v = 0; v < V; v++)
        {
            const float4 u = px[v];
            const float xv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
            for (int j = 0; j < 4; j++)
#pragma unroll
                for (int n = 0; n < 4; n++) acc[n] = fmaf(xv[j], W.k[n * 9 * F + p * F + 4 * v + j], acc[n]);
        }
    }
#pragma unroll
    for (int n = 0; n < 4; n++) row_ptr_w<T>(dst.ptr, dst.pitch, 2 * y + (n >> 1))[2 * x + (n & 1)] = from_float<T>(acc[n]);
}

template <int CIN>
constexpr int stage_bytes()
{
    return SX * SY * CIN * 4;
}

// input tile (+ NB output channels' weights when they go to shared memory)
template <int CIN, int NB>
constexpr int conv_bytes()
{
    return stage_bytes<CIN>() + (kSmemWeights<CIN, NB> ? NB * 9 * CIN * 4 : 0);
}

template <class Kern>
cudaError_t allow_smem(Kern kern, int bytes)
{
    return bytes > 48 * 1024 ? cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) : cudaSuccess;
}

// One 3x3 F->F layer (two launches of 16 output channels for F = 32).
template <int F, int ACT, bool RES>
cudaError_t conv_layer(const float* k, const float* b, const float* a, const float* in, float* out, const float* skip, int w, int h,
                       cudaStream_t stream)
{
    constexpr int NB = F > 16 ? 16 : F;
    const dim3 grid((w + BX - 1) / BX, (h + BY - 1) / BY);
    cudaError_t err = allow_smem(conv_kernel<F, NB, ACT, RES>, conv_bytes<F, NB>());
    if (err != cudaSuccess) return err;
    for (int n0 = 0; n0 < F; n0 += NB)
    {
        ConvW<F, NB> W;
        for (int n = 0; n < NB; n++)
        {
            for (int i = 0; i < 9 * F; i++) W.k[n * 9 * F + i] = k[(n0 + n) * 9 * F + i];
            W.b[n] = b[n0 + n];
            W.a[n] = a ? a[n0 + n] : 0.0f;
        }
        conv_kernel<F, NB, ACT, RES><<<grid, THREADS, conv_bytes<F, NB>(), stream>>>(W, in, out, skip, F, n0, w, h);
        count_launch();
    }
    return cudaGetLastError();
}

template <typename T, int F>
cudaError_t up_layer(const float* k, const float* b, const float* in, const Plane& out, int w, int h, cudaStream_t stream)
{
    const dim3 grid((w + BX - 1) / BX, (h + BY - 1) / BY);
    UpW<F> W;
    for (int i = 0; i < 4 * 9 * F; i++) W.k[i] = k[i];
    for (int i = 0; i < 4; i++) W.b[i] = b[i];
    cudaError_t err = allow_smem(up_kernel<T, F>, stage_bytes<F>());
    if (err != cudaSuccess) return err;
    up_kernel<T, F><<<grid, THREADS, stage_bytes<F>(), stream>>>(W, in, out, w, h);
    count_launch();
    return cudaGetLastError();
}

template <typename T, int K, int F>
cudaError_t head_layer(const float* k, const float* b, const Plane& in, float* feat, cudaStream_t stream)
{
    const dim3 grid((in.w + BX - 1) / BX, (in.h + BY - 1) / BY);
    HeadW<K, F> W;
    for (int i = 0; i < F * K * K; i++) W.k[i] = k[i];
    for (int i = 0; i < F; i++) W.b[i] = b[i];
    head_kernel<T, K, F><<<grid, THREADS, 0, stream>>>(W, in, feat);
    count_launch();
    return cudaGetLastError();
}

template <typename T, int F>
cudaError_t artcnn_typed(const float* kernels, const float* biases, int blocks, const Plane& in, const Plane& out,
                         float* const maps[3], cudaStream_t stream)
{
    const int w = in.w, h = in.h;
    float* feat = maps[0];
    float* a = maps[1];
    float* b = maps[2];
    cudaError_t err = head_layer<T, 3, F>(kernels, biases, in, feat, stream);
    if (err != cudaSuccess) return err;
    const float* cur = feat;
    int l = 1;
    for (int i = 0; i < blocks; i++, l++)
    {
        err = conv_layer<F, kReLU, false>(kernels + F * 9 + F * F * 9 * (l - 1), biases + F * l, nullptr, cur, a, nullptr, w, h,
                                          stream);
        if (err != cudaSuccess) return err;
        cur = a;
        float* t = a;
        a = b;
        b = t;
    }
    err = conv_layer<F, kIdentity, true>(kernels + F * 9 + F * F * 9 * (l - 1), biases + F * l, nullptr, cur, a, feat, w, h,
                                         stream);
    if (err != cudaSuccess) return err;
    l++;
    return up_layer<T, F>(kernels + F * 9 + F * F * 9 * (l - 1), biases + F * l, a, out, w, h, stream);
}

template <typename T, int F>
cudaError_t fsrcnnx_typed(const float* kernels, const float* biases, const float* alphas, int blocks, const Plane& in,
                          const Plane& out, float* const maps[3], cudaStream_t stream)
{
    const int w = in.w, h = in.h;
    float* feat = maps[0];
    float* a = maps[1];
    float* b = maps[2];
    cudaError_t err = head_layer<T, 5, F>(kernels, biases, in, feat, stream);
    if (err != cudaSuccess) return err;
    const float* cur = feat;
    int l = 1;
    for (; l < blocks; l++)
    {
        err = conv_layer<F, kPReLU, false>(kernels + F * 25 + F * F * 9 * (l - 1), biases + F * l, alphas + F * (l - 1), cur, a,
                                           nullptr, w, h, stream);
        if (err != cudaSuccess) return err;
        cur = a;
        float* t = a;
        a = b;
        b = t;
    }
    {
        TailW<F> W;
        const float* k3 = kernels + F * 25 + F * F * 9 * (l - 1);
        for (int i = 0; i < F * 9 * F; i++) W.c3.k[i] = k3[i];
        for (int i = 0; i < F; i++)
        {
            W.c3.b[i] = biases[F * l + i];
            W.c3.a[i] = alphas[F * (l - 1) + i];
            W.b1[i] = biases[F * (l + 1) + i];
            W.a1[i] = alphas[F * l + i];
        }
        for (int i = 0; i < F * F; i++) W.k1[i] = kernels[F * 25 + F * F * 9 * blocks + i];
        err = allow_smem(tail_kernel<F>, conv_bytes<F, F>());
        if (err != cudaSuccess) return err;
        const dim3 grid((w + BX - 1) / BX, (h + BY - 1) / BY);
        tail_kernel<F><<<grid, THREADS, conv_bytes<F, F>(), stream>>>(W, cur, feat, a, w, h);
        count_launch();
        if ((err = cudaGetLastError()) != cudaSuccess) return err;
        l += 2;
    }
    return up_layer<T, F>(kernels + F * 25 + F * F * 9 * blocks + F * F, biases + F * l, a, out, w, h, stream);
}

}  // namespace f3

cudaError_t launch_artcnn_fp32(const float* kernels, const float* biases, int F, int blocks, const Plane& in, const Plane& out,
                               float* const maps[3], cudaStream_t stream)
{
    using namespace f3;
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    if (blocks < 1) return cudaErrorInvalidValue;
    switch (in.type)
    {
    case kU8: return F == 32 ? artcnn_typed<uint8_t, 32>(kernels, biases, blocks, in, out, maps, stream)
                             : artcnn_typed<uint8_t, 16>(kernels, biases, blocks, in, out, maps, stream);
    case kU16: return F == 32 ? artcnn_typed<uint16_t, 32>(kernels, biases, blocks, in, out, maps, stream)
                              : artcnn_typed<uint16_t, 16>(kernels, biases, blocks, in, out, maps, stream);
    case kF32: return F == 32 ? artcnn_typed<float, 32>(kernels, biases, blocks, in, out, maps, stream)
                              : artcnn_typed<float, 16>(kernels, biases, blocks, in, out, maps, stream);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_fsrcnnx_fp32(const float* kernels, const float* biases, const float* alphas, int F, int blocks,
                                const Plane& in, const Plane& out, float* const maps[3], cudaStream_t stream)
{
    using namespace f3;
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    if (blocks < 2) return cudaErrorInvalidValue;
    switch (in.type)
    {
    case kU8: return F == 16 ? fsrcnnx_typed<uint8_t, 16>(kernels, biases, alphas, blocks, in, out, maps, stream)
                             : fsrcnnx_typed<uint8_t, 8>(kernels, biases, alphas, blocks, in, out, maps, stream);
    case kU16: return F == 16 ? fsrcnnx_typed<uint16_t, 16>(kernels, biases, alphas, blocks, in, out, maps, stream)
                              : fsrcnnx_typed<uint16_t, 8>(kernels, biases, alphas, blocks, in, out, maps, stream);
    case kF32: return F == 16 ? fsrcnnx_typed<float, 16>(kernels, biases, alphas, blocks, in, out, maps, stream)
                              : fsrcnnx_typed<float, 8>(kernels, biases, alphas, blocks, in, out, maps, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace acgb
