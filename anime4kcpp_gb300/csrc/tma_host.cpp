// Host-side TMA tensor-map encoding through the driver entry point (no link
// against libcuda: the function is looked up at run time).
#include "tma_host.hpp"

#include <cudaTypedefs.h>

#include <mutex>

namespace acgb {

namespace {

PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

}  // namespace

bool tma_plane_ok(const void* base, int pitch)
{
    return (reinterpret_cast<uintptr_t>(base) & 15u) == 0 && (pitch & 15) == 0 && encoder() != nullptr;
}

bool encode_tmap_2d(CUtensorMap* map, const void* base, int elem_bytes, int dim_x, int dim_y, int pitch, int box_x, int box_y)
{
    auto fn = encoder();
    if (!fn || !tma_plane_ok(base, pitch)) return false;
    CUtensorMapDataType dt = elem_bytes == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                             : (elem_bytes == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32);
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(dim_x), static_cast<cuuint64_t>(dim_y)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(pitch)};
    cuuint32_t box[2] = {static_cast<cuuint32_t>(box_x), static_cast<cuuint32_t>(box_y)};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, dt, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

bool encode_tmap_3d_u16(CUtensorMap* map, const void* base, int d0, int d1, int d2, int b0, int b1, int b2)
{
    return encode_tmap_3d_u16_strided(map, base, d0, d1, d2, b0, b1, b2, 1);
}

bool encode_tmap_3d_u16_strided(CUtensorMap* map, const void* base, int d0, int d1, int d2, int b0, int b1, int b2, int s1)
{
    auto fn = encoder();
    if (!fn || (reinterpret_cast<uintptr_t>(base) & 15u) != 0 || (d0 * 2) % 16 != 0 || (b0 * 2) % 16 != 0) return false;
    cuuint64_t dims[3] = {static_cast<cuuint64_t>(d0), static_cast<cuuint64_t>(d1), static_cast<cuuint64_t>(d2)};
    cuuint64_t strides[2] = {static_cast<cuuint64_t>(d0) * 2, static_cast<cuuint64_t>(d0) * d1 * 2};
    cuuint32_t box[3] = {static_cast<cuuint32_t>(b0), static_cast<cuuint32_t>(b1), static_cast<cuuint32_t>(b2)};
    if (s1 < 1 || s1 > 8) return false;
    cuuint32_t estr[3] = {1, static_cast<cuuint32_t>(s1), 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace acgb
