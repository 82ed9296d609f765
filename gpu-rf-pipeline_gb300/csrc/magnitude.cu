// Magnitude of cf32 samples: mag[i] = |x[i]| (src/magnitude.cu:1-25, tools/reference.py:98-100).
//
// HBM-bound elementwise pass: 12 bytes per sample (8 read, 4 written). A thread takes two
// samples per step (one 16-byte load, one 8-byte store), in a grid-stride loop over a grid of a
// few blocks per SM; an odd last sample is done on its own.
#include "magnitude.cuh"

namespace rfx {
namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
magnitude_kernel(const float4* __restrict__ x, float2* __restrict__ mag, long long pairs,
                 long long n)
{
    const long long stride = static_cast<long long>(gridDim.x) * kThreads;
    for (long long i = static_cast<long long>(blockIdx.x) * kThreads + threadIdx.x; i < pairs;
         i += stride) {
        const float4 v = __ldcs(x + i);   // read once: streaming
        __stcs(mag + i, make_float2(cmag(v.x, v.y), cmag(v.z, v.w)));
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && 2 * pairs < n) {
        const float2 v = reinterpret_cast<const float2*>(x)[n - 1];
        reinterpret_cast<float*>(mag)[n - 1] = cmag(v.x, v.y);
    }
}

}  // namespace

cudaError_t magnitude_launch(const void* x, float* mag, long long n, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    int device = 0;
    int sms = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess) {
        return err;
    }
    const long long pairs = n / 2;
    const long long want = (pairs + kThreads - 1) / kThreads;
    const long long cap = static_cast<long long>(sms) * 8;
    const int grid = static_cast<int>(want < 1 ? 1 : (want < cap ? want : cap));
    magnitude_kernel<<<grid, kThreads, 0, stream>>>(static_cast<const float4*>(x),
                                                     reinterpret_cast<float2*>(mag), pairs, n);
    return cudaGetLastError();
}

}  // namespace rfx
