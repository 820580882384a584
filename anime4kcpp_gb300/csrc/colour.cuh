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

// Both phases of the horizontal pass for source column i of one region row
// (outputs 2i and 2i + 1): taps i .. i + 4 decoded once, each sum ascending as
// in chroma_hpass.  h_out receives 2 x UC floats (phase 0, then phase 1).
template <typename T, int UC>
__device__ __forceinline__ void chroma_hpass2(const T* uv_row, int i, const Phase2& ph, float* h_out)
{
    float d[5][UC];
    if constexpr (sizeof(T) == 1 && UC == 2)
    {
        // the row's UV pairs are 2-byte aligned: one 16-bit load per tap
        const uint16_t* p = reinterpret_cast<const uint16_t*>(uv_row) + i;
#pragma unroll
        for (int t = 0; t < 5; t++)
        {
            const uint32_t v = p[t];
            d[t][0] = decode_float<T>(static_cast<T>(v & 0xFFu));
            d[t][1] = decode_float<T>(static_cast<T>(v >> 8));
        }
    }
    else
    {
#pragma unroll
        for (int t = 0; t < 5; t++)
#pragma unroll
            for (int c = 0; c < UC; c++) d[t][c] = decode_float<T>(uv_row[(i + t) * UC + c]);
    }
    float o[2 * UC];
#pragma unroll
    for (int k = 0; k < 2; k++)
#pragma unroll
        for (int c = 0; c < UC; c++)
        {
            float s = 0.0f;
#pragma unroll
            for (int t = 0; t < 4; t++) s = __fadd_rn(s, __fmul_rn(ph.w[k][t], d[k + t][c]));
            o[k * UC + c] = s;
        }
    if constexpr (UC == 2)
        *reinterpret_cast<float4*>(h_out) = make_float4(o[0], o[1], o[2], o[3]);  // 16-byte aligned (2i even)
    else
    {
#pragma unroll
        for (int c = 0; c < 2 * UC; c++) h_out[c] = o[c];
    }
}

// Bytes of one output row's two pixels (2 x C elements of T) written at `dst`:
// with `wide` (the row start is aligned to the widest store used) in 2-3
// aligned stores, else element by element.
template <typename T, int C>
__device__ __forceinline__ void store_px2(T* dst, const T (&v)[2 * C], bool wide)
{
    if (wide)
    {
        if constexpr (sizeof(T) == 1 && C == 3)
        {
            // 6 bytes at a 2-byte aligned address (6 x is even)
            const uint32_t b01 = v[0] | (v[1] << 8), b23 = v[2] | (v[3] << 8), b45 = v[4] | (v[5] << 8);
            if ((reinterpret_cast<uintptr_t>(dst) & 3u) == 0)
            {
                *reinterpret_cast<uint32_t*>(dst) = b01 | (b23 << 16);
                *reinterpret_cast<uint16_t*>(dst + 4) = static_cast<uint16_t>(b45);
            }
            else
            {
                *reinterpret_cast<uint16_t*>(dst) = static_cast<uint16_t>(b01);
                *reinterpret_cast<uint32_t*>(dst + 2) = b23 | (b45 << 16);
            }
            return;
        }
        else if constexpr (sizeof(T) == 1 && C == 4)
        {
            *reinterpret_cast<uint2*>(dst) = make_uint2(v[0] | (v[1] << 8) | (v[2] << 16) | (static_cast<uint32_t>(v[3]) << 24),
                                                        v[4] | (v[5] << 8) | (v[6] << 16) | (static_cast<uint32_t>(v[7]) << 24));
            return;
        }
        else if constexpr (sizeof(T) == 2 && C == 3)
        {
            uint32_t* d = reinterpret_cast<uint32_t*>(dst);
            d[0] = v[0] | (static_cast<uint32_t>(v[1]) << 16);
            d[1] = v[2] | (static_cast<uint32_t>(v[3]) << 16);
            d[2] = v[4] | (static_cast<uint32_t>(v[5]) << 16);
            return;
        }
        else if constexpr (sizeof(T) == 2 && C == 4)
        {
            uint2* d = reinterpret_cast<uint2*>(dst);
            d[0] = make_uint2(v[0] | (static_cast<uint32_t>(v[1]) << 16), v[2] | (static_cast<uint32_t>(v[3]) << 16));
            d[1] = make_uint2(v[4] | (static_cast<uint32_t>(v[5]) << 16), v[6] | (static_cast<uint32_t>(v[7]) << 16));
            return;
        }
        else if constexpr (sizeof(T) == 4)
        {
            float2* d = reinterpret_cast<float2*>(dst);
#pragma unroll
            for (int k = 0; k < C; k++) d[k] = make_float2(v[2 * k], v[2 * k + 1]);
            return;
        }
    }
#pragma unroll
    for (int k = 0; k < 2 * C; k++) dst[k] = v[k];
}

// Alignment of a row start that store_px2 needs for its wide stores.
template <typename T, int C>
__host__ __device__ constexpr unsigned store_px2_align()
{
    return sizeof(T) == 1 ? (C == 3 ? 4u : 8u) : (sizeof(T) == 2 ? (C == 3 ? 4u : 8u) : 8u);
}

// merge_block2_h with the same arithmetic, loading each of the five H rows
// the 2x2 block needs once (both columns and all channels together) and
// storing each output row's two pixels with store_px2.
template <typename T, int C>
__device__ __forceinline__ void merge_block2_hv(const float* H, int hpitch, int i, int j, const Phase2& ph,
                                                const T (&yq)[2][2], T* out0, T* out1, bool wide, const float* lut)
{
    constexpr int UC = C - 1;
    float h[5][2][UC];
#pragma unroll
    for (int t = 0; t < 5; t++)
    {
        const float* row = H + ((j + t) * hpitch + 2 * i) * UC;
        if constexpr (UC == 2)
        {
            const float4 q = *reinterpret_cast<const float4*>(row);  // 16-byte aligned (2i even)
            h[t][0][0] = q.x;
            h[t][0][1] = q.y;
            h[t][1][0] = q.z;
            h[t][1][1] = q.w;
        }
        else
        {
#pragma unroll
            for (int k = 0; k < 2; k++)
#pragma unroll
                for (int c = 0; c < UC; c++) h[t][k][c] = row[k * UC + c];
        }
    }
#pragma unroll
    for (int dy = 0; dy < 2; dy++)
    {
        T px[2 * C];
#pragma unroll
        for (int k = 0; k < 2; k++)
        {
            float q[UC];
#pragma unroll
            for (int c = 0; c < UC; c++)
            {
                float s = 0.0f;
#pragma unroll
                for (int t = 0; t < 3; t++) s = __fadd_rn(s, __fmul_rn(ph.w[dy][t], h[dy + t][k][c]));
                const float m = __fmul_rn(ph.w[dy][3], h[dy + 3][k][c]);
                if constexpr (sizeof(T) < 4) q[c] = to_float_lut<T>(from_unit<T>(add_sat(s, m)), lut);
                else q[c] = to_float_lut<T>(encode_resampled<T>(__fadd_rn(s, m)), lut);
            }
            yuv_to_rgb_store<T, C>(to_float_lut<T>(yq[dy][k], lut), q[0], q[1], C == 4 ? q[2] : 1.0f, px + k * C);
        }
        store_px2<T, C>(dy ? out1 : out0, px, wide);
    }
}

}  // namespace acgb
