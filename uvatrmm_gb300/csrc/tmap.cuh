// Host-side TMA tensor-map construction (cuTensorMapEncodeTiled through the
// runtime's driver entry point, so the library does not link libcuda).
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace uvt {

// 2-D tiled map over a column-major-style matrix whose contiguous dimension
// has `inner` elements and whose other dimension has `outer` elements, with
// `ld_bytes` between consecutive outer indices.  Box = box_inner x box_outer.
// swizzle128: CU_TENSOR_MAP_SWIZZLE_128B (box_inner * elem must be 128 B).
// Returns 0 on success, else a CUresult-like nonzero code.
int make_tmap_2d(CUtensorMap *map, CUtensorMapDataType dtype, int elem_bytes, const void *base, uint64_t inner,
                 uint64_t outer, uint64_t ld_bytes, uint32_t box_inner, uint32_t box_outer, bool swizzle128);

}  // namespace uvt
