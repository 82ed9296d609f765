// Plain channelizer branch-sum kernel (chan_plain.cu): internal launch interface.
#pragma once

#include <cuda_runtime.h>

namespace rfx {

// u (frames * channels cf32, frame-major) = the polyphase branch sums of x, stored in `format`
// (rfx_sample_format: cf32, ci16, ci8; integer components converted on load).
cudaError_t chan_branch_launch(const void* x, const float* taps, void* u, long long frames,
                               int channels, int num_taps, cudaStream_t stream, int format = 0);

// Whether the branch sums of this shape can be computed for a range of frames
// (chan_branch_launch_range): every branch with 8, 16, 24 or 32 taps, cf32 or ci16 input.
bool chan_branch_ranged(int channels, int num_taps, int format);

// Frames frame0 .. frame0 + frames - 1 of the branch sums into u (row 0 = frame frame0), with
// the same bits as chan_branch_launch gives for those frames. x is the whole input.
cudaError_t chan_branch_launch_range(const void* x, const float* taps, void* u,
                                     long long frame0, long long frames, int channels,
                                     int num_taps, cudaStream_t stream, int format = 0);

}  // namespace rfx
