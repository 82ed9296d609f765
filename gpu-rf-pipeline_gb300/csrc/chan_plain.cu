// Plain channelizer: FP32 polyphase branch sums, then cuFFT's batched inverse transform in
// place — the structure of the project's channelize_device (src/channelize.cu:56-72).
//
//   u[t][m] = sum_p h[pM + m] x[tM - pM - m]          (x[i < 0] = 0)
//   z[t][k] = sum_m u[t][m] e^{+2 pi i k m / M}        (cuFFT inverse, unnormalized)
//
// The branch sums use the project's arithmetic (src/channelize.cu:35-46): one fused
// multiply-add per tap, l = m, m + M, ... ascending, stopping at the start of the input, so u is
// bit-identical to its kernel's. One thread per (frame, branch): consecutive threads read
// consecutive (descending) samples and consecutive taps, so every load is coalesced; the I/Q
// pair is one packed f32x2 fused multiply-add.
#include "chan_plain.cuh"
#include "ptx.cuh"

#include <cuda_runtime.h>
#include <cufft.h>

namespace rfx {

namespace {
constexpr int kBranchThreads = 256;
}

__global__ void __launch_bounds__(kBranchThreads)
chan_branch_kernel(const float2* __restrict__ x, const float* __restrict__ taps,
                   float2* __restrict__ u, long long frames, int channels, int num_taps)
{
    const long long idx = static_cast<long long>(blockIdx.x) * kBranchThreads + threadIdx.x;
    if (idx >= frames * channels) {
        return;
    }
    const long long t = idx / channels;
    const int m = static_cast<int>(idx - t * channels);
    const long long newest = t * channels;  // index of x[tM]
    f32x2 acc = 0ull;
    for (int l = m; l < num_taps; l += channels) {
        const long long s = newest - l;
        if (s < 0) {
            break;
        }
        const float h = __ldg(taps + l);
        const float2 v = __ldg(x + s);
        acc = fma2(pack2(h, h), pack2(v.x, v.y), acc);
    }
    u[idx] = unpack2(acc);
}

cudaError_t chan_branch_launch(const void* x, const float* taps, void* u, long long frames,
                               int channels, int num_taps, cudaStream_t stream)
{
    const long long total = frames * channels;
    if (total == 0) {
        return cudaSuccess;
    }
    const long long grid = (total + kBranchThreads - 1) / kBranchThreads;
    chan_branch_kernel<<<static_cast<unsigned>(grid), kBranchThreads, 0, stream>>>(
        static_cast<const float2*>(x), taps, static_cast<float2*>(u), frames, channels,
        num_taps);
    return cudaGetLastError();
}

}  // namespace rfx
