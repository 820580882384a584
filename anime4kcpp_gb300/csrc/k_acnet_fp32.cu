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
//
// RGB(A) inputs take the fused path: the staging step converts the RGB(A)
// window to quantised Y (rgb2yuv) and keeps the UV(A) of the tile plus 2
// pixels in shared memory; the last layer resamples it x2 (Catmull-Rom) and
// merges it with the new luma (yuv2rgb), writing RGB(A) output directly.
#include <cuda_runtime.h>

#include "colour.cuh"
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
constexpr int UVW = TW + 4;          // chroma region: the tile plus 2 pixels each side
constexpr int UVX0 = HALO - 2;       // its origin in window coordinates
template <typename T, int C>
__host__ __device__ constexpr size_t uv_bytes()
{
    return C == 1 ? 0 : ((UVW * UVW * (C - 1) * sizeof(T) + 15) / 16 * 16);
}
template <typename T, int C>
__host__ __device__ constexpr size_t smem_bytes()
{
    return sizeof(Smem) + uv_bytes<T, C>() + 1024;  // + u8 conversion table
}
static_assert(UVW * 2 * TW * 3 * 4 <= sizeof(float4) * 2 * BH * BW, "horizontal chroma sums must fit a feature buffer");

// Fused-colour arguments of the kernel (small; the weights go separately).
struct ColourArgs
{
    Plane in, out;
    Phase2 ph;
};

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
template <typename T, int C>
__device__ __forceinline__ void layer_last(const AcnetLegacyWeights& W, const float4 (*src)[BH][BW], const Plane& out,
                                           const float* H, const float* lut, const Phase2& ph, int gx0, int gy0, int ix0,
                                           int ix1, int iy0, int iy1)
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
        T o[2][2];
#pragma unroll
        for (int dy = 0; dy < 2; dy++)
#pragma unroll
            for (int dx = 0; dx < 2; dx++)
            {
                const int ko = K2 + 8 * (dy * 2 + dx);
                float d = s[0] * W.k[ko];
#pragma unroll
                for (int c = 1; c < 8; c++) d = fmaf(s[c], W.k[ko + c], d);
                o[dy][dx] = from_float<T>(d);
            }
        T* row0 = row_ptr_w<T>(out.ptr, out.pitch, oy) + ox * C;
        T* row1 = row_ptr_w<T>(out.ptr, out.pitch, oy + 1) + ox * C;
        if constexpr (C == 1)
        {
            row0[0] = o[0][0];
            row0[1] = o[0][1];
            row1[0] = o[1][0];
            row1[1] = o[1][1];
        }
        else merge_block2_h<T, C>(H, 2 * TW, wx - HALO, wy - HALO, ph, o, row0, row1, lut);
    }
}

template <typename T, int C>
__global__ void __launch_bounds__(THREADS, 1)
acnet_legacy_fp32_kernel(const __grid_constant__ AcnetLegacyWeights W, const __grid_constant__ ColourArgs A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& S = *reinterpret_cast<Smem*>(smem_raw);
    T* uvs = reinterpret_cast<T*>(smem_raw + sizeof(Smem));
    float* lut = reinterpret_cast<float*>(smem_raw + sizeof(Smem) + uv_bytes<T, C>());
    const Plane& in = A.in;
    const Plane& out = A.out;
    if constexpr (sizeof(T) == 1)
    {
        if (threadIdx.x < 256) lut[threadIdx.x] = __fdiv_rn(static_cast<float>(threadIdx.x), 255.0f);
        __syncthreads();
    }

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
        if constexpr (C == 1) S.inp[wy][wx] = to_float<T>(row_ptr<T>(in.ptr, in.pitch, gy)[gx]);
        else
        {
            // fused split: quantised Y (rgb2yuv) and, near the tile, UV(A)
            const T* px = row_ptr<T>(in.ptr, in.pitch, gy) + gx * C;
            T v[C];
#pragma unroll
            for (int c = 0; c < C; c++) v[c] = px[c];
            T yq, uvq[C - 1];
            rgb_to_yuv_q_lut<T, C>(v, yq, uvq, lut);
            S.inp[wy][wx] = to_float_lut<T>(yq, lut);
            const int ux = wx - UVX0, uy = wy - UVX0;
            if (ux >= 0 && ux < UVW && uy >= 0 && uy < UVW)
            {
#pragma unroll
                for (int c = 0; c < C - 1; c++) uvs[(uy * UVW + ux) * (C - 1) + c] = uvq[c];
            }
        }
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
    float* H = reinterpret_cast<float*>(&S.fa[0][0][0]);  // dead after layer 7
    if constexpr (C > 1)
    {
        // horizontal pass of the x2 chroma resample for the tile (region rows
        // x output columns), shared by the per-pixel vertical passes
        for (int e = threadIdx.x; e < UVW * 2 * TW; e += THREADS)
        {
            const int r = e / (2 * TW), ox = e - r * (2 * TW);
            chroma_hpass<T, C - 1>(uvs + r * UVW * (C - 1), ox >> 1, ox & 1, A.ph, H + e * (C - 1));
        }
        __syncthreads();
    }
    layer_last<T, C>(W, S.fb, out, H, lut, A.ph, gx0, gy0, ix0, ix1, iy0, iy1);
}

}  // namespace fp32

namespace fp32 {
template <typename T, int C>
cudaError_t launch_typed(const AcnetLegacyWeights& wts, const ColourArgs& a, dim3 grid, cudaStream_t stream)
{
    constexpr size_t bytes = smem_bytes<T, C>();
    // one-time set-up per device, thread-safe
    const cudaError_t setup = device_once([] {
        return cudaFuncSetAttribute(acnet_legacy_fp32_kernel<T, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    });
    if (setup != cudaSuccess) return setup;
    acnet_legacy_fp32_kernel<T, C><<<grid, THREADS, bytes, stream>>>(wts, a);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_channels(const AcnetLegacyWeights& wts, const ColourArgs& a, dim3 grid, cudaStream_t stream)
{
    switch (a.in.channels)
    {
    case 1: return launch_typed<T, 1>(wts, a, grid, stream);
    case 3: return launch_typed<T, 3>(wts, a, grid, stream);
    case 4: return launch_typed<T, 4>(wts, a, grid, stream);
    default: return cudaErrorInvalidValue;
    }
}
}  // namespace fp32

cudaError_t launch_acnet_legacy_fp32(const AcnetLegacyWeights& wts, const Plane& in, const Plane& out, const Phase2* phase2,
                                     cudaStream_t stream)
{
    using namespace fp32;
    if (in.w <= 0 || in.h <= 0) return cudaSuccess;
    if (in.channels > 1 && !phase2) return cudaErrorInvalidValue;
    ColourArgs a;
    a.in = in;
    a.out = out;
    if (phase2) a.ph = *phase2;
    dim3 grid((in.w + TW - 1) / TW, (in.h + TH - 1) / TH);
    cudaError_t err;
    switch (in.type)
    {
    case kU8: err = launch_channels<uint8_t>(wts, a, grid, stream); break;
    case kU16: err = launch_channels<uint16_t>(wts, a, grid, stream); break;
    case kF32: err = launch_channels<float>(wts, a, grid, stream); break;
    default: return cudaErrorInvalidValue;
    }
    if (err == cudaSuccess) count_launch();
    return err;
}

}  // namespace acgb
