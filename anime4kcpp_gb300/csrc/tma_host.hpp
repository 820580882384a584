// Host helpers for TMA tensor maps.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace acgb {

// True when a plane can be described by a tensor map: 16-byte aligned base
// and pitch, and the driver offers the encoder.
bool tma_plane_ok(const void* base, int pitch);

// 2-D tiled tensor map over a pitched plane of dim_x elements per row
// (elements of elem_bytes = 1, 2 or 4 bytes) and dim_y rows; box of
// box_x x box_y elements (box_x * elem_bytes a multiple of 16), no swizzle,
// out-of-bounds elements read as zero.
bool encode_tmap_2d(CUtensorMap* map, const void* base, int elem_bytes, int dim_x, int dim_y, int pitch, int box_x, int box_y);

// 3-D tiled tensor map over a dense [d2][d1][d0] array of 16-bit elements
// (d0 * 2 a multiple of 16 bytes); box of b0 x b1 x b2 elements (b0 * 2 a
// multiple of 16), no swizzle, out-of-bounds elements read as zero.
bool encode_tmap_3d_u16(CUtensorMap* map, const void* base, int d0, int d1, int d2, int b0, int b1, int b2);
// The same with a traversal stride s1 along dimension 1: a load starting at
// x fetches elements x, x + s1, ... (ceil(b1 / s1) of them) along it.
bool encode_tmap_3d_u16_strided(CUtensorMap* map, const void* base, int d0, int d1, int d2, int b0, int b1, int b2, int s1);

}  // namespace acgb
