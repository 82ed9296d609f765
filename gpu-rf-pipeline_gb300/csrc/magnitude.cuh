// Magnitude of complex samples (csrc/magnitude.cu) and the expression the fused channelizer
// epilogue shares with it.
#pragma once

#include <cuda_runtime.h>

namespace rfx {

// |z| = sqrt(re^2 + im^2) as the project defines it (src/magnitude.cu:17-25), with the rounding
// steps written out (im^2 rounded, one fused multiply-add, correctly rounded square root) so
// that the standalone kernel and the fused channelizer epilogue give the same bits.
__device__ __forceinline__ float cmag(float re, float im)
{
    return __fsqrt_rn(__fmaf_rn(re, re, __fmul_rn(im, im)));
}

// mag[i] = |x[i]| for i < n; x cf32, 8-byte aligned (16-byte for the vector path), mag float.
cudaError_t magnitude_launch(const void* x, float* mag, long long n, cudaStream_t stream);

}  // namespace rfx
