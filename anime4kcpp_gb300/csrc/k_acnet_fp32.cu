// Plain FP32 layer-fused ACNetLegacy x2 pass (CUDA cores).
//
// Network (core/include/AC/Core/Model/ACNet.hpp:18-61, core/src/Model.cpp:8-35,
// CPU order core/src/processor/cpu/CPUProcessor.cpp:1371-1390):
//   layer 0     conv3x3 1->8 + bias + ReLU            (Common.hpp:166-197)
//   layers 1-7  conv3x3 8->8 + bias + ReLU            (Common.hpp:116-164)
//   layer 8     conv3x3 8->8 + bias + ReLU, then a 2x2 stride-2 transposed
//               conv 8->1 without bias, fromFloat     (Common.hpp:344-393)
// Every 3x3 read is clamped to the edge of the map it reads (the image for
// layer 0, the previous layer's feature map afterwards).
//
// GB300 mapping: one CTA computes a 32x32 tile of input pixels (64x64 output
// pixels) for all nine layers without touching HBM in between.  It stages a
// haloed 50x50 luma window (9-pixel halo = receptive field of nine 3x3
// convolutions) in shared memory as FP32, then runs the layers between two
// ping-pong FP32 feature buffers in shared memory (each 48x48 pixels x 8
// channels, split into two float4 planes so a warp's 16-byte loads of
// consecutive pixels are bank-conflict free).  Layer k computes the window
// inset by k+1 pixels, intersected with the image.  Reads are clamped to the
// positions the previous layer computed inside the image, which is exactly the
// reference's clamp-to-edge on the intermediate map.
//
// Weights are passed by value as a __grid_constant__ kernel parameter (19 KB,
// constant bank 0); every layer is unrolled with compile-time weight offsets
// so each FFMA takes its weight straight from the constant bank.
#include <cuda_runtime.h>

#include "device_common.cuh"
#include "kernels.hpp"

namespace acgb {
namespace fp32 {

constexpr int TW = 32, TH = 32, HALO = 9;
constexpr int WW = TW + 2 * HALO, WH = TH + 2 * HALO;  // input window
constexpr int BW = WW - 2, BH = WH - 2;                // feature buffers (window inset 1)
constexpr int THREADS = 512;

struct Smem
{
    float4 fa[2][BH][BW];
    float4 fb[2][BH][BW];
    float inp[WH][WW];
};
constexpr size_t kSmemBytes = sizeof(Smem);

// Layer 0: 1 -> 8 from the staged input window (edge-replicated at staging,
// which equals clamped reads).
__device__ __forceinline__ void layer0(const AcnetLegacyWeights& W, const Smem& S, float4 (*dst)[BH][BW],
                                       int ix0, int ix1, int iy0, int iy1)
{
    const int rx0 = max(1, ix0), rx1 = min(WW - 2, ix1);
    const int ry0 = max(1, iy0), ry1 = min(WH - 2, iy1);
    const int nx = rx1 - rx0 + 1, ny = ry1 - ry0 + 1;
    if (nx <= 0 || ny <= 0) return;
    for (int i = threadIdx.x; i < nx * ny; i += THREADS)
    {
        const int wy = ry0 + i / nx, wx = rx0 + i % nx;
        float r[9];
#pragma unroll
        for (int ty = 0; ty < 3; ty++)
#pragma unroll
            for (int tx = 0; tx < 3; tx++) r[ty * 3 + tx] = S.inp[wy + ty - 1][wx + tx - 1];
        float acc[8];
#pragma unroll
        for (int n = 0; n < 8; n++)
        {
            float s = r[0] * W.k[n * 9 + 0];
#pragma unroll
            for (int t = 1; t < 9; t++) s = fmaf(r[t], W.k[n * 9 + t], s);
            acc[n] = fmaxf(s + W.b[n], 0.0f);
        }
        dst[0][wy - 1][wx - 1] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        dst[1][wy - 1][wx - 1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
    }
}

// 3x3 conv 8 -> 8 of layer L at window position (wx, wy) with clamped taps.
template <int L>
__device__ __forceinline__ void conv8(const AcnetLegacyWeights& W, const float4 (*src)[BH][BW], int wx, int wy,
                                      int lox, int hix, int loy, int hiy, float acc[8])
{
    constexpr int KO = 72 + 576 * (L - 1);
    const int xs[3] = {max(wx - 1, lox), wx, min(wx + 1, hix)};
    const int ys[3] = {max(wy - 1, loy), wy, min(wy + 1, hiy)};
#pragma unroll
    for (int n = 0; n < 8; n++) acc[n] = 0.0f;
#pragma unroll
    for (int ty = 0; ty < 3; ty++)
    {
#pragma unroll
        for (int tx = 0; tx < 3; tx++)
        {
            const float4 a = src[0][ys[ty] - 1][xs[tx] - 1];
            const float4 b = src[1][ys[ty] - 1][xs[tx] - 1];
            const float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
            const int p = ty * 3 + tx;
#pragma unroll
            for (int n = 0; n < 8; n++)
#pragma unroll
                for (int c = 0; c < 8; c++) acc[n] = fmaf(v[c], W.k[KO + n * 72 + p * 8 + c], acc[n]);
        }
    }
#pragma unroll
    for (int n = 0; n < 8; n++) acc[n] = fmaxf(acc[n] + W.b[8 * L + n], 0.0f);
}

template <int L>
__device__ __forceinline__ void layer8(const AcnetLegacyWeights& W, const float4 (*src)[BH][BW], float4 (*dst)[BH][BW],
                                       int ix0, int ix1, int iy0, int iy1)
{
    const int rx0 = max(L + 1, ix0), rx1 = min(WW - 2 - L, ix1);
    const int ry0 = max(L + 1, iy0), ry1 = min(WH - 2 - L, iy1);
    const int lox = max(L, ix0), hix = min(WW - 1 - L, ix1);
    const int loy = max(L, iy0), hiy = min(WH - 1 - L, iy1);
    const int nx = rx1 - rx0 + 1, ny = ry1 - ry0 + 1;
    if (nx <= 0 || ny <= 0) return;
    for (int i = threadIdx.x; i < nx * ny; i += THREADS)
    {
        const int wy = ry0 + i / nx, wx = rx0 + i % nx;
        float acc[8];
        conv8<L>(W, src, wx, wy, lox, hix, loy, hiy, acc);
        dst[0][wy - 1][wx - 1] = make_float4(acc[0], acc[1], acc[2], acc[3]);
        dst[1][wy - 1][wx - 1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
    }
}

// Layer 8 + deconv 2x2 stride 2 (8 -> 1, no bias) straight to global memory.
template <typename T>
__device__ __forceinline__ void layer_last(const AcnetLegacyWeights& W, const float4 (*src)[BH][BW], const Plane& out,
                                           int gx0, int gy0, int ix0, int ix1, int iy0, int iy1)
{
    constexpr int L = 8;
    constexpr int K2 = 72 + 576 * 8;
    const int rx0 = max(L + 1, ix0), rx1 = min(WW - 2 - L, ix1);
    const int ry0 = max(L + 1, iy0), ry1 = min(WH - 2 - L, iy1);
    const int lox = max(L, ix0), hix = min(WW - 1 - L, ix1);
    const int loy = max(L, iy0), hiy = min(WH - 1 - L, iy1);
    const int nx = rx1 - rx0 + 1, ny = ry1 - ry0 + 1;
    if (nx <= 0 || ny <= 0) return;
    for (int i = threadIdx.x; i < nx * ny; i += THREADS)
    {
        const int wy = ry0 + i / nx, wx = rx0 + i % nx;
        float s[8];
        conv8<L>(W, src, wx, wy, lox, hix, loy, hiy, s);
        const int ox = 2 * (gx0 + wx), oy = 2 * (gy0 + wy);
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
        {
            T o[2];
#pragma unroll
            for (int dx = 0; dx < 2; dx++)
            {
                const int ko = K2 + 8 * (dy * 2 + dx);
                float d = s[0] * W.k[ko];
#pragma unroll
                for (int c = 1; c < 8; c++) d = fmaf(s[c], W.k[ko + c], d);
                o[dx] = from_float<T>(d);
            }
            T* row = row_ptr_w<T>(out.ptr, out.pitch, oy + dy) + ox;
            row[0] = o[0];
            row[1] = o[1];
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(THREADS, 1)
acnet_legacy_fp32_kernel(const __grid_constant__ AcnetLegacyWeights W, const Plane in, const Plane out)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);

    const int gx0 = blockIdx.x * TW - HALO, gy0 = blockIdx.y * TH - HALO;
    // Window range that lies inside the image (inclusive, window coordinates).
    const int ix0 = max(0, -gx0), ix1 = min(WW - 1, in.w - 1 - gx0);
    const int iy0 = max(0, -gy0), iy1 = min(WH - 1, in.h - 1 - gy0);

    // Stage the haloed input window, converting to float once; positions
    // outside the image take the nearest edge value.
    for (int i = threadIdx.x; i < WW * WH; i += THREADS)
    {
        const int wy = i / WW, wx = i % WW;
        const int gx = clampi(gx0 + wx, 0, in.w - 1), gy = clampi(gy0 + wy, 0, in.h - 1);
        S.inp[wy][wx] = to_float<T>(row_ptr<T>(in.ptr, in.pitch, gy)[gx]);
    }
    __syncthreads();
    layer0(W, S, S.fa, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer8<1>(W, S.fa, S.fb, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer8<2>(W, S.fb, S.fa, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer8<3>(W, S.fa, S.fb, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer8<4>(W, S.fb, S.fa, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer8<5>(W, S.fa, S.fb, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer8<6>(W, S.fb, S.fa, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer8<7>(W, S.fa, S.fb, ix0, ix1, iy0, iy1);
    __syncthreads();
    layer_last<T>(W, S.fb, out, gx0, gy0, ix0, ix1, iy0, iy1);
}

}  // namespace fp32

cudaError_t launch_acnet_legacy_fp32(const AcnetLegacyWeights& wts, const Plane& in, const Plane& out, cudaStream_t stream)
{
    using namespace fp32;
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    dim3 grid((in.w + TW - 1) / TW, (in.h + TH - 1) / TH);
    cudaError_t err = cudaSuccess;
    switch (in.type)
    {
    case kU8:
        err = cudaFuncSetAttribute(acnet_legacy_fp32_kernel<uint8_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
        if (err != cudaSuccess) return err;
        acnet_legacy_fp32_kernel<uint8_t><<<grid, THREADS, kSmemBytes, stream>>>(wts, in, out);
        break;
    case kU16:
        err = cudaFuncSetAttribute(acnet_legacy_fp32_kernel<uint16_t>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
        if (err != cudaSuccess) return err;
        acnet_legacy_fp32_kernel<uint16_t><<<grid, THREADS, kSmemBytes, stream>>>(wts, in, out);
        break;
    case kF32:
        err = cudaFuncSetAttribute(acnet_legacy_fp32_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
        if (err != cudaSuccess) return err;
        acnet_legacy_fp32_kernel<float><<<grid, THREADS, kSmemBytes, stream>>>(wts, in, out);
        break;
    default: return cudaErrorInvalidValue;
    }
    count_launch();
    return cudaGetLastError();
}

}  // namespace acgb
