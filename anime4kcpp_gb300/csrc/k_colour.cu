// Colour split / merge and separable resampling kernels.
//
// rgb2yuv / rgba2yuva restate core/src/ImageProcess.cpp:39-61 and :114-138;
// yuv2rgb / yuva2rgba restate :192-215 and :276-308.  The resampler restates
// the filter definitions of core/src/ImageResize.cpp:62-83 (Catmull-Rom),
// :127-134 (bilinear) and point sampling with edge clamp; the reference runs
// them through stb_image_resize2, which this backend does not use.
//
// All of these are memory-bound elementwise kernels: one thread per output
// pixel, consecutive threads on consecutive pixels of a row (coalesced).
// Arithmetic uses explicitly rounded intrinsics so it matches the
// reference's scalar CPU code bit for bit.
#include <atomic>

#include "colour.cuh"
#include "device_common.cuh"
#include "kernels.hpp"

namespace acgb {

namespace {
std::atomic<uint64_t> g_launches{0};
}
uint64_t launch_count() { return g_launches.load(); }
void count_launch(int n) { g_launches.fetch_add(static_cast<uint64_t>(n)); }

template <typename T, int C>
__global__ void rgb2yuv_split_kernel(Plane rgb, Plane yp, Plane uvp)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= rgb.w) return;
    const T* in = row_ptr<T>(rgb.ptr, rgb.pitch, y) + x * C;
    float r = to_float<T>(in[0]);
    float g = to_float<T>(in[1]);
    float b = to_float<T>(in[2]);
    float a = 1.0f;
    if constexpr (C == 4)
    {
        a = to_float<T>(in[3]);
        r = __fmul_rn(r, a);
        g = __fmul_rn(g, a);
        b = __fmul_rn(b, a);
    }
    float yy = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, r), __fmul_rn(0.587f, g)), __fmul_rn(0.114f, b));
    float u = __fadd_rn(__fmul_rn(0.564f, __fsub_rn(b, yy)), 0.5f);
    float v = __fadd_rn(__fmul_rn(0.713f, __fsub_rn(r, yy)), 0.5f);
    row_ptr_w<T>(yp.ptr, yp.pitch, y)[x] = from_float<T>(yy);
    T* uo = row_ptr_w<T>(uvp.ptr, uvp.pitch, y) + x * (C - 1);
    uo[0] = from_float<T>(u);
    uo[1] = from_float<T>(v);
    if constexpr (C == 4) uo[2] = from_float<T>(a);
}

template <typename T, int C>
__global__ void rgb2yuv_packed_kernel(Plane rgb, Plane yuv)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= rgb.w) return;
    const T* in = row_ptr<T>(rgb.ptr, rgb.pitch, y) + x * C;
    float r = to_float<T>(in[0]);
    float g = to_float<T>(in[1]);
    float b = to_float<T>(in[2]);
    float a = 1.0f;
    if constexpr (C == 4)
    {
        a = to_float<T>(in[3]);
        r = __fmul_rn(r, a);
        g = __fmul_rn(g, a);
        b = __fmul_rn(b, a);
    }
    float yy = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, r), __fmul_rn(0.587f, g)), __fmul_rn(0.114f, b));
    float u = __fadd_rn(__fmul_rn(0.564f, __fsub_rn(b, yy)), 0.5f);
    float v = __fadd_rn(__fmul_rn(0.713f, __fsub_rn(r, yy)), 0.5f);
    T* out = row_ptr_w<T>(yuv.ptr, yuv.pitch, y) + x * C;
    out[0] = from_float<T>(yy);
    out[1] = from_float<T>(u);
    out[2] = from_float<T>(v);
    if constexpr (C == 4) out[3] = from_float<T>(a);
}

template <typename T, int C>
__global__ void yuv2rgb_packed_kernel(Plane yuv, Plane rgb)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= yuv.w) return;
    const T* in = row_ptr<T>(yuv.ptr, yuv.pitch, y) + x * C;
    float yy = to_float<T>(in[0]);
    float u = to_float<T>(in[1]);
    float v = to_float<T>(in[2]);
    float a = C == 4 ? to_float<T>(in[3]) : 1.0f;
    yuv_to_rgb_store<T, C>(yy, u, v, a, row_ptr_w<T>(rgb.ptr, rgb.pitch, y) + x * C);
}

// Resampled value of channel `ch` of an interleaved plane at output (ox, oy):
// horizontal sums per source row (ascending taps), then the vertical sum,
// all in float with explicit rounding; zero weights skipped.
template <typename T, int NC>
__device__ __forceinline__ float resample(const Plane& src, const ResizeAxis& ax, const ResizeAxis& ay, int ox, int oy, int ch)
{
    const int fx = ax.first[ox];
    const int fy = ay.first[oy];
    const float* wxs = ax.w + static_cast<size_t>(ox) * ax.taps;
    const float* wys = ay.w + static_cast<size_t>(oy) * ay.taps;
    float s = 0.0f;
    for (int j = 0; j < ay.taps; j++)
    {
        float wy = wys[j];
        if (wy == 0.0f) continue;
        int sy = clampi(fy + j, 0, src.h - 1);
        const T* row = row_ptr<T>(src.ptr, src.pitch, sy);
        float hsum = 0.0f;
        for (int i = 0; i < ax.taps; i++)
        {
            float wx = wxs[i];
            if (wx == 0.0f) continue;
            int sx = clampi(fx + i, 0, src.w - 1);
            hsum = __fadd_rn(hsum, __fmul_rn(wx, decode_float<T>(row[sx * NC + ch])));
        }
        s = __fadd_rn(s, __fmul_rn(wy, hsum));
    }
    return s;
}

template <typename T, int C>
__global__ void merge_resize_kernel(Plane yp, Plane uvp, ResizeAxis ax, ResizeAxis ay, Plane rgb)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= yp.w) return;
    constexpr int UC = C - 1;
    float yy = to_float<T>(row_ptr<T>(yp.ptr, yp.pitch, y)[x]);
    // resample, quantise to the element type (the reference stores the
    // resized UV as an image of the source type), then normalise again.
    float u = to_float<T>(encode_resampled<T>(resample<T, UC>(uvp, ax, ay, x, y, 0)));
    float v = to_float<T>(encode_resampled<T>(resample<T, UC>(uvp, ax, ay, x, y, 1)));
    float a = 1.0f;
    if constexpr (C == 4) a = to_float<T>(encode_resampled<T>(resample<T, UC>(uvp, ax, ay, x, y, 2)));
    yuv_to_rgb_store<T, C>(yy, u, v, a, row_ptr_w<T>(rgb.ptr, rgb.pitch, y) + x * C);
}

// Integer-factor merge: the chroma plane (W x H) is resampled by exactly F on
// both axes.  Output o = F*i + k samples source taps i + off[k] .. + 3 with
// weights w[k][0..3] (phase k only), so one thread per source pixel computes
// its F x F output block: horizontal sums for the rows it needs once, then the
// vertical sums -- the same operations, in the same order, as the separable
// table-driven path (horizontal pass per source row, ascending taps, then the
// vertical pass), so the results are identical.
template <int F>
struct PhaseTable
{
    float w[F][4];
};

// First source tap of output phase k relative to the source index i:
// ceil((k + 0.5) / F - 2.5) for the support-2 Catmull-Rom filter.
template <int F>
__host__ __device__ constexpr int phase_off(int k)
{
    return F == 2 ? (k == 0 ? -2 : -1) : (k < F / 2 ? -2 : -1);
}

// The integer-factor resample alone (a planar chroma plane of the video
// recipe): the same phase-table sums as merge_int_kernel, each output
// encoded to the plane's element type.  One thread per source pixel writes
// its F x F block of NC-channel outputs.
template <typename T, int NC, int F>
__global__ void resize_int_kernel(Plane src, PhaseTable<F> tab, Plane dst)
{
    const int sx = blockIdx.x * blockDim.x + threadIdx.x;
    const int sy = blockIdx.y;
    if (sx >= src.w) return;
    constexpr int RLO = -2, NR = 5;  // source rows sy-2 .. sy+2 cover every phase
    float h[NR][F][NC];
#pragma unroll
    for (int rr = 0; rr < NR; rr++)
    {
        const T* row = row_ptr<T>(src.ptr, src.pitch, clampi(sy + RLO + rr, 0, src.h - 1));
        T v[5][NC];
#pragma unroll
        for (int dx = 0; dx < 5; dx++)
        {
            const int xs = clampi(sx - 2 + dx, 0, src.w - 1);
#pragma unroll
            for (int c = 0; c < NC; c++) v[dx][c] = row[xs * NC + c];
        }
#pragma unroll
        for (int k = 0; k < F; k++)
#pragma unroll
            for (int c = 0; c < NC; c++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 4; t++)
                {
                    const float wt = tab.w[k][t];
                    if (wt == 0.0f) continue;
                    s = __fadd_rn(s, __fmul_rn(wt, decode_float<T>(v[phase_off<F>(k) + t + 2][c])));
                }
                h[rr][k][c] = s;
            }
    }
#pragma unroll
    for (int j = 0; j < F; j++)
    {
        T* orow = row_ptr_w<T>(dst.ptr, dst.pitch, F * sy + j) + F * sx * NC;
#pragma unroll
        for (int k = 0; k < F; k++)
#pragma unroll
            for (int c = 0; c < NC; c++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 4; t++)
                {
                    const float wt = tab.w[j][t];
                    if (wt == 0.0f) continue;
                    s = __fadd_rn(s, __fmul_rn(wt, h[phase_off<F>(j) + t - RLO][k][c]));
                }
                orow[k * NC + c] = encode_resampled<T>(s);
            }
    }
}

template <typename T, int C, int F>
__global__ void merge_int_kernel(Plane yp, Plane uvp, PhaseTable<F> tab, Plane rgb)
{
    const int sx = blockIdx.x * blockDim.x + threadIdx.x;
    const int sy = blockIdx.y;
    if (sx >= uvp.w) return;
    constexpr int UC = C - 1;
    constexpr int RLO = -2, NR = 5;  // source rows sy-2 .. sy+2 cover every phase
    float h[NR][F][UC];
#pragma unroll
    for (int rr = 0; rr < NR; rr++)
    {
        const T* row = row_ptr<T>(uvp.ptr, uvp.pitch, clampi(sy + RLO + rr, 0, uvp.h - 1));
        T v[5][UC];
#pragma unroll
        for (int dx = 0; dx < 5; dx++)
        {
            const int xs = clampi(sx - 2 + dx, 0, uvp.w - 1);
#pragma unroll
            for (int c = 0; c < UC; c++) v[dx][c] = row[xs * UC + c];
        }
#pragma unroll
        for (int k = 0; k < F; k++)
#pragma unroll
            for (int c = 0; c < UC; c++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 4; t++)
                {
                    const float wt = tab.w[k][t];
                    if (wt == 0.0f) continue;
                    s = __fadd_rn(s, __fmul_rn(wt, decode_float<T>(v[phase_off<F>(k) + t + 2][c])));
                }
                h[rr][k][c] = s;
            }
    }
#pragma unroll
    for (int j = 0; j < F; j++)
    {
        const int oy = F * sy + j;
        const T* yrow = row_ptr<T>(yp.ptr, yp.pitch, oy);
        T* orow = row_ptr_w<T>(rgb.ptr, rgb.pitch, oy);
#pragma unroll
        for (int k = 0; k < F; k++)
        {
            float uvv[UC];
#pragma unroll
            for (int c = 0; c < UC; c++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 4; t++)
                {
                    const float wt = tab.w[j][t];
                    if (wt == 0.0f) continue;
                    s = __fadd_rn(s, __fmul_rn(wt, h[phase_off<F>(j) + t - RLO][k][c]));
                }
                uvv[c] = to_float<T>(encode_resampled<T>(s));
            }
            const int ox = F * sx + k;
            const float yy = to_float<T>(yrow[ox]);
            yuv_to_rgb_store<T, C>(yy, uvv[0], uvv[1], C == 4 ? uvv[2] : 1.0f, orow + ox * C);
        }
    }
}

template <typename T, int NC>
__global__ void resize_kernel(Plane src, Plane dst, ResizeAxis ax, ResizeAxis ay)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    int y = blockIdx.y;
    if (x >= dst.w) return;
    T* out = row_ptr_w<T>(dst.ptr, dst.pitch, y) + x * NC;
    for (int c = 0; c < NC; c++) out[c] = encode_resampled<T>(resample<T, NC>(src, ax, ay, x, y, c));
}

// Element-wise shift of an integer plane, shl / shr of
// core/src/ImageProcess.cpp:601-616: n > 0 shifts left, n < 0 right; the
// result is stored back in the element type (a left shift drops high bits).
// In place when src and dst are the same plane.
template <typename T>
__device__ __forceinline__ T shift_one(unsigned v, int n)
{
    return static_cast<T>(n >= 0 ? (v << n) : (v >> (-n)));
}
template <typename T>
__global__ void shift_kernel(Plane src, Plane dst, int n)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= src.w * src.channels) return;
    const unsigned v = row_ptr<T>(src.ptr, src.pitch, y)[x];
    row_ptr_w<T>(dst.ptr, dst.pitch, y)[x] = shift_one<T>(v, n);
}
// The same with 16 bytes per thread, for planes whose base addresses and
// pitches are 16-byte aligned: thread x of a row takes elements
// [x * E, x * E + E) (E = 16 / sizeof(T)); the row's last partial chunk
// goes element by element.
template <typename T>
__global__ void shift16_kernel(Plane src, Plane dst, int n)
{
    constexpr int E = 16 / static_cast<int>(sizeof(T));
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    const int elems = src.w * src.channels, x0 = x * E;
    if (x0 >= elems) return;
    const T* in = row_ptr<T>(src.ptr, src.pitch, y) + x0;
    T* out = row_ptr_w<T>(dst.ptr, dst.pitch, y) + x0;
    if (x0 + E <= elems)
    {
        uint4 v = *reinterpret_cast<const uint4*>(in);
        T* e = reinterpret_cast<T*>(&v);
#pragma unroll
        for (int k = 0; k < E; k++) e[k] = shift_one<T>(e[k], n);
        *reinterpret_cast<uint4*>(out) = v;
    }
    else
        for (int k = 0; x0 + k < elems; k++) out[k] = shift_one<T>(in[k], n);
}

namespace {

dim3 row_grid(int w, int h, int block) { return dim3((w + block - 1) / block, h); }

}  // namespace

#define ACGB_TYPE_SWITCH(type, ...)                     \
    switch (type)                                       \
    {                                                   \
    case kU8: { using T = uint8_t; __VA_ARGS__ } break;  \
    case kU16: { using T = uint16_t; __VA_ARGS__ } break; \
    case kF32: { using T = float; __VA_ARGS__ } break;   \
    default: return cudaErrorInvalidValue;              \
    }

cudaError_t launch_rgb2yuv_split(const Plane& rgb, const Plane& y, const Plane& uv, cudaStream_t stream)
{
    if (rgb.w <= 0 || rgb.h <= 0) return cudaSuccess;
    dim3 grid = row_grid(rgb.w, rgb.h, 128);
    ACGB_TYPE_SWITCH(rgb.type,
        if (rgb.channels == 4) rgb2yuv_split_kernel<T, 4><<<grid, 128, 0, stream>>>(rgb, y, uv);
        else rgb2yuv_split_kernel<T, 3><<<grid, 128, 0, stream>>>(rgb, y, uv);)
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_rgb2yuv_packed(const Plane& rgb, const Plane& yuv, cudaStream_t stream)
{
    if (rgb.w <= 0 || rgb.h <= 0) return cudaSuccess;
    dim3 grid = row_grid(rgb.w, rgb.h, 128);
    ACGB_TYPE_SWITCH(rgb.type,
        if (rgb.channels == 4) rgb2yuv_packed_kernel<T, 4><<<grid, 128, 0, stream>>>(rgb, yuv);
        else rgb2yuv_packed_kernel<T, 3><<<grid, 128, 0, stream>>>(rgb, yuv);)
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_yuv2rgb_packed(const Plane& yuv, const Plane& rgb, cudaStream_t stream)
{
    if (yuv.w <= 0 || yuv.h <= 0) return cudaSuccess;
    dim3 grid = row_grid(yuv.w, yuv.h, 128);
    ACGB_TYPE_SWITCH(yuv.type,
        if (yuv.channels == 4) yuv2rgb_packed_kernel<T, 4><<<grid, 128, 0, stream>>>(yuv, rgb);
        else yuv2rgb_packed_kernel<T, 3><<<grid, 128, 0, stream>>>(yuv, rgb);)
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_merge_resize(const Plane& y, const Plane& uv, ResizeAxis ax, ResizeAxis ay, const Plane& rgb,
                                cudaStream_t stream)
{
    if (y.w <= 0 || y.h <= 0) return cudaSuccess;
    dim3 grid = row_grid(y.w, y.h, 128);
    ACGB_TYPE_SWITCH(y.type,
        if (rgb.channels == 4) merge_resize_kernel<T, 4><<<grid, 128, 0, stream>>>(y, uv, ax, ay, rgb);
        else merge_resize_kernel<T, 3><<<grid, 128, 0, stream>>>(y, uv, ax, ay, rgb);)
    count_launch();
    return cudaGetLastError();
}

template <int F>
static cudaError_t launch_merge_int_f(const Plane& y, const Plane& uv, const float* wx, const Plane& rgb, cudaStream_t stream)
{
    PhaseTable<F> tab;
    for (int k = 0; k < F; k++)
        for (int t = 0; t < 4; t++) tab.w[k][t] = wx[k * 4 + t];
    dim3 grid = row_grid(uv.w, uv.h, 128);
    ACGB_TYPE_SWITCH(y.type,
        if (rgb.channels == 4) merge_int_kernel<T, 4, F><<<grid, 128, 0, stream>>>(y, uv, tab, rgb);
        else merge_int_kernel<T, 3, F><<<grid, 128, 0, stream>>>(y, uv, tab, rgb);)
    count_launch();
    return cudaGetLastError();
}

int merge_int_phase_offset(int factor, int k) { return factor == 2 ? phase_off<2>(k) : phase_off<4>(k); }

template <int F>
static cudaError_t launch_resize_int_f(const Plane& src, const Plane& dst, const float* wx, cudaStream_t stream)
{
    PhaseTable<F> tab;
    for (int k = 0; k < F; k++)
        for (int t = 0; t < 4; t++) tab.w[k][t] = wx[k * 4 + t];
    dim3 grid = row_grid(src.w, src.h, 128);
    ACGB_TYPE_SWITCH(src.type,
        switch (src.channels)
        {
        case 1: resize_int_kernel<T, 1, F><<<grid, 128, 0, stream>>>(src, tab, dst); break;
        case 2: resize_int_kernel<T, 2, F><<<grid, 128, 0, stream>>>(src, tab, dst); break;
        case 3: resize_int_kernel<T, 3, F><<<grid, 128, 0, stream>>>(src, tab, dst); break;
        case 4: resize_int_kernel<T, 4, F><<<grid, 128, 0, stream>>>(src, tab, dst); break;
        default: return cudaErrorInvalidValue;
        })
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_resize_int(const Plane& src, const Plane& dst, int factor, const float* phase_weights,
                              cudaStream_t stream)
{
    if (src.w <= 0 || src.h <= 0) return cudaSuccess;
    if (dst.w != factor * src.w || dst.h != factor * src.h || dst.channels != src.channels || dst.type != src.type)
        return cudaErrorInvalidValue;
    if (factor == 2) return launch_resize_int_f<2>(src, dst, phase_weights, stream);
    if (factor == 4) return launch_resize_int_f<4>(src, dst, phase_weights, stream);
    return cudaErrorInvalidValue;
}

cudaError_t launch_merge_int(const Plane& y, const Plane& uv, int factor, const float* phase_weights, const Plane& rgb,
                             cudaStream_t stream)
{
    if (uv.w <= 0 || uv.h <= 0) return cudaSuccess;
    if (factor == 2) return launch_merge_int_f<2>(y, uv, phase_weights, rgb, stream);
    if (factor == 4) return launch_merge_int_f<4>(y, uv, phase_weights, rgb, stream);
    return cudaErrorInvalidValue;
}

cudaError_t launch_shift(const Plane& src, const Plane& dst, int n, cudaStream_t stream)
{
    if (src.w <= 0 || src.h <= 0 || n == 0) return cudaSuccess;
    if (n <= -16 || n >= 16) return cudaErrorInvalidValue;
    const bool vec = ((reinterpret_cast<uintptr_t>(src.ptr) | reinterpret_cast<uintptr_t>(dst.ptr) |
                       static_cast<uintptr_t>(src.pitch) | static_cast<uintptr_t>(dst.pitch)) & 15) == 0;
    if (vec && (src.type == kU8 || src.type == kU16))
    {
        const int es = src.type & 0xff;
        const int chunks = (src.w * src.channels * es + 15) / 16;
        const dim3 g = row_grid(chunks, src.h, 256);
        if (src.type == kU8) shift16_kernel<uint8_t><<<g, 256, 0, stream>>>(src, dst, n);
        else shift16_kernel<uint16_t><<<g, 256, 0, stream>>>(src, dst, n);
        count_launch();
        return cudaGetLastError();
    }
    dim3 grid = row_grid(src.w * src.channels, src.h, 256);
    switch (src.type)
    {
    case kU8: shift_kernel<uint8_t><<<grid, 256, 0, stream>>>(src, dst, n); break;
    case kU16: shift_kernel<uint16_t><<<grid, 256, 0, stream>>>(src, dst, n); break;
    default: return cudaErrorInvalidValue;
    }
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_resize(const Plane& src, const Plane& dst, ResizeAxis ax, ResizeAxis ay, cudaStream_t stream)
{
    if (dst.w <= 0 || dst.h <= 0) return cudaSuccess;
    dim3 grid = row_grid(dst.w, dst.h, 128);
    ACGB_TYPE_SWITCH(src.type,
        switch (src.channels)
        {
        case 1: resize_kernel<T, 1><<<grid, 128, 0, stream>>>(src, dst, ax, ay); break;
        case 2: resize_kernel<T, 2><<<grid, 128, 0, stream>>>(src, dst, ax, ay); break;
        case 3: resize_kernel<T, 3><<<grid, 128, 0, stream>>>(src, dst, ax, ay); break;
        case 4: resize_kernel<T, 4><<<grid, 128, 0, stream>>>(src, dst, ax, ay); break;
        default: return cudaErrorInvalidValue;
        })
    count_launch();
    return cudaGetLastError();
}

}  // namespace acgb
