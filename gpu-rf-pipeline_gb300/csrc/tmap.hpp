// Tensor-map (TMA descriptor) encoding for the kernels, through the runtime's driver entry
// point query (no link against libcuda).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace rfx {

// A 2-D float32 view of `base`: `rows` rows of `row_floats` floats each (row stride
// 4 * row_floats bytes), copied in boxes of box_x floats by box_y rows; reads outside the view
// return zeros. base must be 16-byte aligned and 4 * row_floats a multiple of 16.
cudaError_t encode_rows_f32(CUtensorMap* map, const void* base, long long rows, int row_floats,
                            unsigned box_x, unsigned box_y);

// The same view over elements of `elem_bytes` bytes (4: float32, 2: int16, 1: int8 / raw bytes):
// the copy moves the bits, zero outside the view. elem_bytes * row_elems a multiple of 16.
cudaError_t encode_rows(CUtensorMap* map, const void* base, int elem_bytes, long long rows,
                        int row_elems, unsigned box_x, unsigned box_y);

}  // namespace rfx
