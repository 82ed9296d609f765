// Tensor-core channelizer for 1024 channels (chan_wide.cu): internal launch interface.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

namespace rfx {

// The form takes 1024 channels, any tap count and every sample format (the branch sums are
// chan_branch_launch's).
bool chan_wide_supported(int channels);
// Device bytes of the plan's image (the 32-point DFT operand, hi and lo, and the 1024-point
// twiddles, from FP64) and the kernel that builds it.
size_t chan_wide_image_bytes();
cudaError_t chan_wide_build_image(void* img, cudaStream_t stream);
// z: frames x 1024 cf32 (frame-major); with `magnitude`, frames x 1024 float |z|. u: scratch
// of frames x 1024 cf32 for the branch sums. x in `format` (rfx_sample_format).
cudaError_t chan_wide_launch(const void* x, const float* taps, const void* image, void* u,
                             void* z, long long n, int num_taps, cudaStream_t stream,
                             bool magnitude, int format);
cudaError_t chan_wide_take_fault(unsigned int* code);

}  // namespace rfx
