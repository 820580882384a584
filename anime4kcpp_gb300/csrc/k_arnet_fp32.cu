// ARNet<8> x2 pass, plain FP32, one kernel per layer.
//
// Network (core/include/AC/Core/Model/ARNet.hpp:16-72; CPU order
// core/src/processor/cpu/CPUProcessor.cpp:1464-1491; layer templates
// core/internal/AC/Core/Internal/Processor/CPU/Common.hpp:116-197,223-342):
//   head      conv3x3 1->8, identity                          -> feat
//   block 1   conv3x3 8->8 + PReLU; conv3x3 8->8, out = 0.2*conv + feat
//   block i   conv3x3 8->8 + PReLU; conv3x3 8->8, out = 0.2*conv + block input
//   block B   conv3x3 8->8 + PReLU; conv3x3 8->8 (0.2*conv + block input), then
//             conv1x1 8->8 + PReLU + feat                      (fused, one kernel)
//   upscale   conv3x3 8->4, pixel shuffle 2x2, + toFloat(input pixel), fromFloat
// All 3x3 reads clamp to the map's edge.
//
// The receptive field grows with depth (2B+2 pixels), so the layers are not
// fused into one window: each layer reads and writes an 8-channel FP32 map
// in HBM ([h][w][8], 32 bytes per pixel).  A block of 256 threads computes a
// 32x8 pixel tile from a haloed 34x10 tile staged in shared memory as two
// float4 planes (conflict-free 16-byte loads); each thread computes one
// pixel's 8 outputs (576 FFMA) with the layer's weights taken from the
// constant bank (a by-value kernel parameter).
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.hpp"

namespace acgb {
namespace arnet {

constexpr int BX = 32, BY = 8, THREADS = BX * BY;
constexpr int SX = BX + 2, SY = BY + 2;

struct Conv8W
{
    float k[576];
    float b[8];
    float a[8];  // PReLU slopes (unused for identity layers)
};
struct TailW
{
    Conv8W c3;     // 3x3 identity + residual
    float k1[64];  // 1x1 8->8
    float b1[8];
    float a1[8];   // PReLU of the 1x1
};
struct HeadW
{
    float k[72];
    float b[8];
    float a[8];  // PReLU slopes (ACNet<8> head; unused for ARNet's identity head)
};
struct UpW
{
    float k[288];
    float b[4];
};

enum Act { kIdentity = 0, kPReLU = 1 };

__device__ __forceinline__ float prelu(float v, float a)
{
    // max(v, 0) + a * min(v, 0) (Common.hpp:43-50)
    return fmaxf(v, 0.0f) + a * fminf(v, 0.0f);
}

// Stage the 34x10 haloed tile of an 8-channel map (clamped) into smem.
__device__ __forceinline__ void stage(float4 (*s)[SY][SX], const float* in, int w, int h, int x0, int y0)
{
    for (int i = threadIdx.x; i < SX * SY; i += THREADS)
    {
        const int sy = i / SX, sx = i % SX;
        const int gx = clampi(x0 - 1 + sx, 0, w - 1), gy = clampi(y0 - 1 + sy, 0, h - 1);
        const float4* p = reinterpret_cast<const float4*>(in + (static_cast<size_t>(gy) * w + gx) * 8);
        s[0][sy][sx] = p[0];
        s[1][sy][sx] = p[1];
    }
}

template <int ACT, bool RES>
__global__ void __launch_bounds__(THREADS) conv8_kernel(const __grid_constant__ Conv8W W, const float* __restrict__ in,
                                                        float* __restrict__ out, const float* __restrict__ skip,
                                                        float scale, int w, int h)
{
    __shared__ float4 s[2][SY][SX];
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    stage(s, in, w, h, x0, y0);
    __syncthreads();
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= w || y >= h) return;
    float acc[8];
#pragma unroll
    for (int n = 0; n < 8; n++) acc[n] = W.b[n];
#pragma unroll
    for (int p = 0; p < 9; p++)
    {
        const float4 u = s[0][ty + p / 3][tx + p % 3];
        const float4 v = s[1][ty + p / 3][tx + p % 3];
        const float xv[8] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w};
#pragma unroll
        for (int n = 0; n < 8; n++)
#pragma unroll
            for (int c = 0; c < 8; c++) acc[n] = fmaf(xv[c], W.k[n * 72 + p * 8 + c], acc[n]);
    }
    const size_t o = (static_cast<size_t>(y) * w + x) * 8;
    float r[8];
#pragma unroll
    for (int n = 0; n < 8; n++)
    {
        float v = ACT == kPReLU ? prelu(acc[n], W.a[n]) : acc[n];
        if (RES) v = fmaf(v, scale, skip[o + n]);
        r[n] = v;
    }
    reinterpret_cast<float4*>(out + o)[0] = make_float4(r[0], r[1], r[2], r[3]);
    reinterpret_cast<float4*>(out + o)[1] = make_float4(r[4], r[5], r[6], r[7]);
}

// Last block's second conv (identity, 0.2 residual) fused with the 1x1 conv
// + PReLU + feat (Common.hpp:223-288).
__global__ void __launch_bounds__(THREADS) tail_kernel(const __grid_constant__ TailW W, const float* __restrict__ in,
                                                       const float* __restrict__ skip, const float* __restrict__ feat,
                                                       float* __restrict__ out, float scale, int w, int h)
{
    __shared__ float4 s[2][SY][SX];
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    stage(s, in, w, h, x0, y0);
    __syncthreads();
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= w || y >= h) return;
    float acc[8];
#pragma unroll
    for (int n = 0; n < 8; n++) acc[n] = W.c3.b[n];
#pragma unroll
    for (int p = 0; p < 9; p++)
    {
        const float4 u = s[0][ty + p / 3][tx + p % 3];
        const float4 v = s[1][ty + p / 3][tx + p % 3];
        const float xv[8] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w};
#pragma unroll
        for (int n = 0; n < 8; n++)
#pragma unroll
            for (int c = 0; c < 8; c++) acc[n] = fmaf(xv[c], W.c3.k[n * 72 + p * 8 + c], acc[n]);
    }
    const size_t o = (static_cast<size_t>(y) * w + x) * 8;
    float buf[8];
#pragma unroll
    for (int n = 0; n < 8; n++) buf[n] = fmaf(acc[n], scale, skip[o + n]);
    float r[8];
#pragma unroll
    for (int n = 0; n < 8; n++)
    {
        float v = W.b1[n];
#pragma unroll
        for (int c = 0; c < 8; c++) v = fmaf(buf[c], W.k1[n * 8 + c], v);
        r[n] = prelu(v, W.a1[n]) + feat[o + n];
    }
    reinterpret_cast<float4*>(out + o)[0] = make_float4(r[0], r[1], r[2], r[3]);
    reinterpret_cast<float4*>(out + o)[1] = make_float4(r[4], r[5], r[6], r[7]);
}

// Head: conv3x3 1->8 from the input plane, identity (ARNet) or PReLU
// (ACNet<8>).
template <typename T, int ACT>
__global__ void __launch_bounds__(THREADS) head_kernel(const __grid_constant__ HeadW W, Plane in, float* __restrict__ feat)
{
    __shared__ float s[SY][SX];
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    for (int i = threadIdx.x; i < SX * SY; i += THREADS)
    {
        const int sy = i / SX, sx = i % SX;
        const int gx = clampi(x0 - 1 + sx, 0, in.w - 1), gy = clampi(y0 - 1 + sy, 0, in.h - 1);
        s[sy][sx] = to_float<T>(row_ptr<T>(in.ptr, in.pitch, gy)[gx]);
    }
    __syncthreads();
    const int tx = threadIdx.x % BX, ty = threadIdx.x / BX;
    const int x = x0 + tx, y = y0 + ty;
    if (x >= in.w || y >= in.h) return;
    float r[8];
#pragma unroll
    for (int n = 0; n < 8; n++)
    {
        float v = W.b[n];
#pragma unroll
        for (int p = 0; p < 9; p++) v = fmaf(s[ty + p / 3][tx + p % 3], W.k[n * 9 + p], v);
        r[n] = ACT == kPReLU ? prelu(v, W.a[n]) : v;
    }
    float* o = feat + (static_cast<size_t>(y) * in.w + x) * 8;
    reinterpret_cast<float4*>(o)[0] = make_float4(r[0], r[1], r[2], r[3]);
    reinterpret_cast<float4*>(o)[1] = make_float4(r[4], r[5], r[6], r[7]);
}

// Upscale: conv3x3 8->4 (identity), pixel shuffle, + nearest input, fromFloat.
template <typename T>
__global__ void __launch_bounds__(THREADS) up_kernel(const __grid_constant__ UpW W, const float* __restrict__ in, Plane src,
                                                     Plane dst)
{
    __shared__ float4 s[2][SY][SX];
    const int w = src.w, h = src.h;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    stage(s, in, w, h, x0, y0);
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
        const float4 u = s[0][ty + p / 3][tx + p % 3];
        const float4 v = s[1][ty + p / 3][tx + p % 3];
        const float xv[8] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w};
#pragma unroll
        for (int n = 0; n < 4; n++)
#pragma unroll
            for (int c = 0; c < 8; c++) acc[n] = fmaf(xv[c], W.k[n * 72 + p * 8 + c], acc[n]);
    }
    const float near = to_float<T>(row_ptr<T>(src.ptr, src.pitch, y)[x]);
#pragma unroll
    for (int n = 0; n < 4; n++) row_ptr_w<T>(dst.ptr, dst.pitch, 2 * y + (n >> 1))[2 * x + (n & 1)] = from_float<T>(acc[n] + near);
}

}  // namespace arnet

// Runs one ARNet x2 pass.  maps: four [h][w][8] FP32 work maps.
cudaError_t launch_arnet_fp32(const float* kernels, const float* biases, const float* alphas, int blocks, const Plane& in,
                              const Plane& out, float* const maps[4], cudaStream_t stream)
{
    using namespace arnet;
    const int w = in.w, h = in.h;
    if (w <= 0 || h <= 0) return cudaSuccess;
    if (blocks < 2) return cudaErrorInvalidValue;
    dim3 grid((w + BX - 1) / BX, (h + BY - 1) / BY);
    float* feat = maps[0];
    float* t1 = maps[1];
    float* t2 = maps[2];
    float* t3 = maps[3];
    auto koff = [](int l) { return l <= 0 ? 0 : 72 + 576 * (l - 1); };
    auto aoff = [](int l) { return 8 * ((l - 1) / 2); };
    auto conv_w = [&](int l, bool act) {
        Conv8W W;
        for (int i = 0; i < 576; i++) W.k[i] = kernels[koff(l) + i];
        for (int i = 0; i < 8; i++) W.b[i] = biases[8 * l + i];
        for (int i = 0; i < 8; i++) W.a[i] = act ? alphas[aoff(l) + i] : 0.0f;
        return W;
    };
    int launches = 0;
    {
        HeadW W;
        for (int i = 0; i < 72; i++) W.k[i] = kernels[i];
        for (int i = 0; i < 8; i++) W.b[i] = biases[i];
        for (int i = 0; i < 8; i++) W.a[i] = 0.0f;
        switch (in.type)
        {
        case kU8: head_kernel<uint8_t, kIdentity><<<grid, THREADS, 0, stream>>>(W, in, feat); break;
        case kU16: head_kernel<uint16_t, kIdentity><<<grid, THREADS, 0, stream>>>(W, in, feat); break;
        case kF32: head_kernel<float, kIdentity><<<grid, THREADS, 0, stream>>>(W, in, feat); break;
        default: return cudaErrorInvalidValue;
        }
        launches++;
    }
    int l = 1;
    conv8_kernel<kPReLU, false><<<grid, THREADS, 0, stream>>>(conv_w(l, true), feat, t1, nullptr, 0.0f, w, h);
    l++;
    conv8_kernel<kIdentity, true><<<grid, THREADS, 0, stream>>>(conv_w(l, false), t1, t2, feat, 0.2f, w, h);
    l++;
    launches += 2;
    for (int i = 0; i < blocks - 2; i++)
    {
        conv8_kernel<kPReLU, false><<<grid, THREADS, 0, stream>>>(conv_w(l, true), t2, t1, nullptr, 0.0f, w, h);
        l++;
        conv8_kernel<kIdentity, true><<<grid, THREADS, 0, stream>>>(conv_w(l, false), t1, t3, t2, 0.2f, w, h);
        l++;
        float* t = t2;
        t2 = t3;
        t3 = t;
        launches += 2;
    }
    conv8_kernel<kPReLU, false><<<grid, THREADS, 0, stream>>>(conv_w(l, true), t2, t1, nullptr, 0.0f, w, h);
    l++;
    launches++;
    {
        TailW W;
        W.c3 = conv_w(l, false);
        for (int i = 0; i < 64; i++) W.k1[i] = kernels[72 + 576 * (2 * blocks) + i];
        for (int i = 0; i < 8; i++) W.b1[i] = biases[8 * (l + 1) + i];
        for (int i = 0; i < 8; i++) W.a1[i] = alphas[8 * blocks + i];
        tail_kernel<<<grid, THREADS, 0, stream>>>(W, t1, t2, feat, t3, 0.2f, w, h);
        l += 2;
        launches++;
    }
    {
        UpW W;
        for (int i = 0; i < 288; i++) W.k[i] = kernels[72 + 576 * (2 * blocks) + 64 + i];
        for (int i = 0; i < 4; i++) W.b[i] = biases[8 * l + i];
        switch (in.type)
        {
        case kU8: up_kernel<uint8_t><<<grid, THREADS, 0, stream>>>(W, t3, in, out); break;
        case kU16: up_kernel<uint16_t><<<grid, THREADS, 0, stream>>>(W, t3, in, out); break;
        case kF32: up_kernel<float><<<grid, THREADS, 0, stream>>>(W, t3, in, out); break;
        default: return cudaErrorInvalidValue;
        }
        launches++;
    }
    count_launch(launches);
    return cudaGetLastError();
}

// Runs one ACNet<8> x2 pass (core/include/AC/Core/Model/ACNet.hpp:63-116, CPU
// order core/src/processor/cpu/CPUProcessor.cpp:1417-1436): head conv3x3
// 1->8 + PReLU, `blocks` x conv3x3 8->8 + PReLU, then the upscale layer of
// ARNet (conv3x3 8->4, pixel shuffle, + nearest input).  Weight offsets
// ACNet.hpp:93-114: layer l's kernels at 72 + 576 (l - 1), biases at 8 l,
// slopes at 8 l.  maps: two [h][w][8] FP32 work maps.
cudaError_t launch_acnet8_fp32(const float* kernels, const float* biases, const float* alphas, int blocks, const Plane& in,
                               const Plane& out, float* const maps[2], cudaStream_t stream)
{
    using namespace arnet;
    const int w = in.w, h = in.h;
    if (w <= 0 || h <= 0) return cudaSuccess;
    if (blocks < 1) return cudaErrorInvalidValue;
    dim3 grid((w + BX - 1) / BX, (h + BY - 1) / BY);
    float* a = maps[0];
    float* b = maps[1];
    {
        HeadW W;
        for (int i = 0; i < 72; i++) W.k[i] = kernels[i];
        for (int i = 0; i < 8; i++) W.b[i] = biases[i];
        for (int i = 0; i < 8; i++) W.a[i] = alphas[i];
        switch (in.type)
        {
        case kU8: head_kernel<uint8_t, kPReLU><<<grid, THREADS, 0, stream>>>(W, in, a); break;
        case kU16: head_kernel<uint16_t, kPReLU><<<grid, THREADS, 0, stream>>>(W, in, a); break;
        case kF32: head_kernel<float, kPReLU><<<grid, THREADS, 0, stream>>>(W, in, a); break;
        default: return cudaErrorInvalidValue;
        }
    }
    for (int l = 1; l <= blocks; l++)
    {
        Conv8W W;
        for (int i = 0; i < 576; i++) W.k[i] = kernels[72 + 576 * (l - 1) + i];
        for (int i = 0; i < 8; i++) W.b[i] = biases[8 * l + i];
        for (int i = 0; i < 8; i++) W.a[i] = alphas[8 * l + i];
        conv8_kernel<kPReLU, false><<<grid, THREADS, 0, stream>>>(W, a, b, nullptr, 0.0f, w, h);
        float* t = a;
        a = b;
        b = t;
    }
    {
        UpW W;
        for (int i = 0; i < 288; i++) W.k[i] = kernels[72 + 576 * blocks + i];
        for (int i = 0; i < 4; i++) W.b[i] = biases[8 * (blocks + 1) + i];
        switch (in.type)
        {
        case kU8: up_kernel<uint8_t><<<grid, THREADS, 0, stream>>>(W, a, in, out); break;
        case kU16: up_kernel<uint16_t><<<grid, THREADS, 0, stream>>>(W, a, in, out); break;
        case kF32: up_kernel<float><<<grid, THREADS, 0, stream>>>(W, a, in, out); break;
        default: return cudaErrorInvalidValue;
        }
    }
    count_launch(blocks + 2);
    return cudaGetLastError();
}

}  // namespace acgb
