// Tensor-core channelizer (chan_tc.cu): internal launch interface.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

namespace rfx {

bool chan_tc_supported(int channels, int num_taps);
// Device bytes of the twiddle operand image, and the kernel that builds it (FP64 twiddles).
size_t chan_tc_twiddle_bytes();
cudaError_t chan_tc_build_twiddles(void* img, cudaStream_t stream);
// z: frames x 64 cf32; with `magnitude`, frames x 64 float |z| (the fused epilogue). x in
// `format` (rfx_sample_format: cf32, ci16, ci8), converted where the kernel reads it.
cudaError_t chan_tc_launch(const void* x, const float* taps, const void* twiddles, void* z,
                           long long n, int num_taps, cudaStream_t stream,
                           bool magnitude = false, int format = 0);
cudaError_t chan_tc_take_fault(unsigned int* code);

}  // namespace rfx
