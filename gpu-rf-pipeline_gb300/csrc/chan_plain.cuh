// Plain channelizer branch-sum kernel (chan_plain.cu): internal launch interface.
#pragma once

#include <cuda_runtime.h>

namespace rfx {

// u (frames * channels cf32, frame-major) = the polyphase branch sums of x, stored in `format`
// (rfx_sample_format: cf32, ci16, ci8; integer components converted on load).
cudaError_t chan_branch_launch(const void* x, const float* taps, void* u, long long frames,
                               int channels, int num_taps, cudaStream_t stream, int format = 0);

}  // namespace rfx
