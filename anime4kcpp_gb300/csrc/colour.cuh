// Device colour conversion and the x2 Catmull-Rom chroma resample, shared by
// the standalone colour kernels and the fused prologue/epilogue of the
// layer-fused CNN kernels.
//
// rgb2yuv / rgba2yuva: core/src/ImageProcess.cpp:39-61, :114-138 (Y and UV(A)
// re-quantised to the source element type); yuv2rgb / yuva2rgba: :192-215,
// :276-308.  All roundings follow the reference's scalar code (no fused
// multiply-add), so results are bit-identical to its CPU processor.
#pragma once

#include "device_common.cuh"
#include "kernels.hpp"

namespace acgb {

// RGB(A) pixel -> quantised Y and UV(A) of the same element type.
template <typename T, int C>
__device__ __forceinline__ void rgb_to_yuv_q(const T* in, T& yq, T* uvq)
{
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
    const float yy = __fadd_rn(__fadd_rn(__fmul_rn(0.299f, r), __fmul_rn(0.587f, g)), __fmul_rn(0.114f, b));
    const float u = __fadd_rn(__fmul_rn(0.564f, __fsub_rn(b, yy)), 0.5f);
    const float v = __fadd_rn(__fmul_rn(0.713f, __fsub_rn(r, yy)), 0.5f);
    yq = from_float<T>(yy);
    uvq[0] = from_float<T>(u);
    uvq[1] = from_float<T>(v);
    if constexpr (C == 4) uvq[2] = from_float<T>(a);
}

// yuv2rgb on normalised inputs; writes C channels.
template <typename T, int C>
__device__ __forceinline__ void yuv_to_rgb_store(float yy, float u, float v, float a, T* out)
{
    u = __fsub_rn(u, 0.5f);
    v = __fsub_rn(v, 0.5f);
    if constexpr (C == 3 && sizeof(T) < 4)
    {
        // integer RGB: the saturation folded into the last rounded operation
        out[0] = from_unit<T>(add_sat(yy, __fmul_rn(1.403f, v)));
        out[1] = from_unit<T>(sub_sat(__fsub_rn(yy, __fmul_rn(0.344f, u)), __fmul_rn(0.714f, v)));
        out[2] = from_unit<T>(add_sat(yy, __fmul_rn(1.773f, u)));
        return;
    }
    float r = __fadd_rn(yy, __fmul_rn(1.403f, v));
    float g = __fsub_rn(__fsub_rn(yy, __fmul_rn(0.344f, u)), __fmul_rn(0.714f, v));
    float b = __fadd_rn(yy, __fmul_rn(1.773f, u));
    if constexpr (C == 4)
    {
        if (a > 1e-6f)
        {
            r = __fdiv_rn(r, a);
            g = __fdiv_rn(g, a);
            b = __fdiv_rn(b, a);
        }
        else r = g = b = 0.0f;
    }
    out[0] = from_float<T>(r);
    out[1] = from_float<T>(g);
    out[2] = from_float<T>(b);
    if constexpr (C == 4) out[3] = from_float<T>(a);
}

// toFloat through a table of the 256 u8 values (built with IEEE division, so
// identical to to_float<uint8_t>); other types convert directly.
template <typename T>
__device__ __forceinline__ float to_float_lut(T v, const float* lut)
{
    if constexpr (sizeof(T) == 1) return lut[v];
    else return to_float<T>(v);
}

template <typename T, int C>
__device__ __forceinline__ void rgb_to_yuv_q_lut(const T* in, T& yq, T* uvq, const float* lut)
{
    float r = to_float_lut<T>(in[0], lut);
    float g = to_float_lut<T>(in[1], lut);
    float b = to_float_lut<T>(in[2], lut);
    float a = 1.0f;
    if constexpr (C == 4)
    {
        a = to_float_lut<T>(in[3], lut);
        r = __fmul_rn(r, a);
        g = __fmul_rn(g, a);
        b = __fmul_rn(b, a);
    }
    const float ry = __fadd_rn(__fmul_rn(0.299f, r), __fmul_rn(0.587f, g));
    const float yy = __fadd_rn(ry, __fmul_rn(0.114f, b));
    if constexpr (sizeof(T) < 4)
    {
        // integer outputs: the saturation folded into the last rounded add
        // (an input alpha is already in [0, 1])
        yq = from_unit<T>(add_sat(ry, __fmul_rn(0.114f, b)));
        uvq[0] = from_unit<T>(add_sat(__fmul_rn(0.564f, __fsub_rn(b, yy)), 0.5f));
        uvq[1] = from_unit<T>(add_sat(__fmul_rn(0.713f, __fsub_rn(r, yy)), 0.5f));
        if constexpr (C == 4) uvq[2] = from_unit<T>(a);
    }
    else
    {
        const float u = __fadd_rn(__fmul_rn(0.564f, __fsub_rn(b, yy)), 0.5f);
        const float v = __fadd_rn(__fmul_rn(0.713f, __fsub_rn(r, yy)), 0.5f);
        yq = from_float<T>(yy);
        uvq[0] = from_float<T>(u);
        uvq[1] = from_float<T>(v);
        if constexpr (C == 4) uvq[2] = from_float<T>(a);
    }
}

// Horizontal pass of the x2 chroma resample for one region row: for output
// column ox = 2*i + k (i = tile-local source column), the weighted sum of
// region columns i + k .. i + k + 3 (the region starts two pixels left of the
// tile), ascending.  H receives UC floats per output column.
template <typename T, int UC>
__device__ __forceinline__ void chroma_hpass(const T* uv_row, int i, int k, const Phase2& ph, float* h_out)
{
#pragma unroll
    for (int c = 0; c < UC; c++)
    {
        float s = 0.0f;
#pragma unroll
        for (int t = 0; t < 4; t++) s = __fadd_rn(s, __fmul_rn(ph.w[k][t], decode_float<T>(uv_row[(i + k + t) * UC + c])));
        h_out[c] = s;
    }
}

// Vertical pass + merge for the 2x2 outputs of tile-local source pixel
// (i, j): H holds the horizontal sums, rows = region rows (region row 0 is two
// rows above the tile), hpitch output columns per row, UC floats each.
template <typename T, int C>
__device__ __forceinline__ void merge_block2_h(const float* H, int hpitch, int i, int j, const Phase2& ph, const T (&yq)[2][2],
                                               T* out0, T* out1, const float* lut)
{
    constexpr int UC = C - 1;
#pragma unroll
    for (int dy = 0; dy < 2; dy++)
    {
        T* out = dy ? out1 : out0;
#pragma unroll
        for (int k = 0; k < 2; k++)
        {
            float q[UC];
#pragma unroll
            for (int c = 0; c < UC; c++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 3; t++)
                    s = __fadd_rn(s, __fmul_rn(ph.w[dy][t], H[((j + dy + t) * hpitch + 2 * i + k) * UC + c]));
                const float m = __fmul_rn(ph.w[dy][3], H[((j + dy + 3) * hpitch + 2 * i + k) * UC + c]);
                if constexpr (sizeof(T) < 4) q[c] = to_float_lut<T>(from_unit<T>(add_sat(s, m)), lut);
                else q[c] = to_float_lut<T>(encode_resampled<T>(__fadd_rn(s, m)), lut);
            }
            yuv_to_rgb_store<T, C>(to_float_lut<T>(yq[dy][k], lut), q[0], q[1], C == 4 ? q[2] : 1.0f, out + k * C);
        }
    }
}

// The 2x2 output block of source pixel (cx, cy): luma yq[dy][dx] (already
// quantised) merged with the chroma of a UV(A) region `uv` (UC channels of
// type T per pixel, `pitch` pixels per row; (cx, cy) in region coordinates
// with two pixels of neighbourhood available on every side).  Horizontal
// sums per source row first (ascending taps), then vertical sums: the same
// operations, in the same order, as the separable resampler.
template <typename T, int C>
__device__ __forceinline__ void merge_block2(const T* uv, int pitch, int cx, int cy, const Phase2& ph, const T (&yq)[2][2],
                                             T* out0, T* out1)
{
    constexpr int UC = C - 1;
    float h[5][2][UC];
#pragma unroll
    for (int rr = 0; rr < 5; rr++)
    {
        const T* row = uv + ((cy - 2 + rr) * pitch + (cx - 2)) * UC;
#pragma unroll
        for (int c = 0; c < UC; c++)
        {
            float d[5];
#pragma unroll
            for (int i = 0; i < 5; i++) d[i] = decode_float<T>(row[i * UC + c]);
#pragma unroll
            for (int k = 0; k < 2; k++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 4; t++) s = __fadd_rn(s, __fmul_rn(ph.w[k][t], d[k + t]));
                h[rr][k][c] = s;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < 2; j++)
    {
        T* out = j ? out1 : out0;
#pragma unroll
        for (int k = 0; k < 2; k++)
        {
            float q[UC];
#pragma unroll
            for (int c = 0; c < UC; c++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 4; t++) s = __fadd_rn(s, __fmul_rn(ph.w[j][t], h[j + t][k][c]));
                q[c] = to_float<T>(encode_resampled<T>(s));
            }
            yuv_to_rgb_store<T, C>(to_float<T>(yq[j][k]), q[0], q[1], C == 4 ? q[2] : 1.0f, out + k * C);
        }
    }
}

}  // namespace acgb
