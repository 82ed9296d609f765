// Tensor-core FIR on CTA pairs (fir_tc2.cu): internal interface.
#pragma once

#include <cuda_runtime.h>

namespace rfx {

// Whether the pair kernel takes this tap count (its shared-memory layout fits).
bool fir_tc2_supported(int num_taps);

// n >= 256 samples; `stages` caps the operand ring depth (2, 4 or 6; the largest that fits).
cudaError_t fir_tc2_launch(const void* x, const float* taps, void* y, long long n, int num_taps,
                           int stages, cudaStream_t stream);
cudaError_t fir_tc2_take_fault(unsigned int* code);

}  // namespace rfx
