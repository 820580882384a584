// Device-side helpers shared by the kernels of the GB300 upscaling backend.
//
// Element types follow the reference's ac::core::Image encoding
// (core/include/AC/Core/Image.hpp:365-370): (kind << 8) | bytes.
//
// toFloat/fromFloat restate core/internal/AC/Core/Internal/Util.hpp:50-78.
// Every rounding step of the reference's scalar code is reproduced with
// explicitly rounded intrinsics (__fmul_rn / __fadd_rn / __fdiv_rn) so that
// the compiler cannot contract them into fused multiply-adds; the results are
// then bit-identical to the reference's x86 build for the colour conversion,
// the resize and the quantisation steps.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace acgb {

enum ElemType : int { kU8 = 0x001, kU16 = 0x002, kF32 = 0x204 };

template <typename T> struct TypeMax;
template <> struct TypeMax<uint8_t> { static constexpr float value = 255.0f; };
template <> struct TypeMax<uint16_t> { static constexpr float value = 65535.0f; };

// Util.hpp:50-61: unsigned -> v / max (IEEE division), float as is.
template <typename T>
__device__ __forceinline__ float to_float(T v)
{
    if constexpr (sizeof(T) == 4) return v;
    else return __fdiv_rn(static_cast<float>(v), TypeMax<T>::value);
}

// Util.hpp:63-78: saturate to [0, 1]; unsigned -> (T)(s * max + 0.5f).
template <typename T>
__device__ __forceinline__ T from_float(float v)
{
    float s = v < 0.0f ? 0.0f : (v < 1.0f ? v : 1.0f);
    if constexpr (sizeof(T) == 4) return s;
    else return static_cast<T>(__float2uint_rz(__fadd_rn(__fmul_rn(s, TypeMax<T>::value), 0.5f)));
}

// Rounded add / subtract / fused multiply-add whose result is clamped to
// [0, 1] (PTX .sat).  For non-NaN values this equals rounding and then
// applying fromFloat's saturation, so fromFloat of such a result needs only
// the scaling (from_unit).
__device__ __forceinline__ float add_sat(float a, float b)
{
    float r;
    asm("add.rn.sat.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float sub_sat(float a, float b)
{
    float r;
    asm("sub.rn.sat.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float fma_sat(float a, float b, float c)
{
    float r;
    asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// fromFloat of a value already in [0, 1]: (T)(s * max + 0.5f) for unsigned
// types, s for float.
template <typename T>
__device__ __forceinline__ T from_unit(float s)
{
    if constexpr (sizeof(T) == 4) return s;
    else return static_cast<T>(__float2uint_rz(__fadd_rn(__fmul_rn(s, TypeMax<T>::value), 0.5f)));
}

// The resampler's decode (multiplication by the reciprocal of the maximum).
template <typename T>
__device__ __forceinline__ float decode_float(T v)
{
    if constexpr (sizeof(T) == 4) return v;
    else return __fmul_rn(static_cast<float>(v), 1.0f / TypeMax<T>::value);
}

// The resampler's encode: integer outputs via from_float, float outputs raw.
template <typename T>
__device__ __forceinline__ T encode_resampled(float v)
{
    if constexpr (sizeof(T) == 4) return v;
    else return from_float<T>(v);
}

template <typename T>
__device__ __forceinline__ const T* row_ptr(const void* base, int pitch, int y)
{
    return reinterpret_cast<const T*>(static_cast<const uint8_t*>(base) + static_cast<size_t>(pitch) * y);
}
template <typename T>
__device__ __forceinline__ T* row_ptr_w(void* base, int pitch, int y)
{
    return reinterpret_cast<T*>(static_cast<uint8_t*>(base) + static_cast<size_t>(pitch) * y);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace acgb
