// Plain FP32 FIR kernels for sm_103a: one tile of 2304 outputs per block of 256 threads
// (fir_plain_tile.cuh holds the tile function, its arithmetic and its staging), for one capture,
// for captures sharing one tap set, for captures with their own taps, and for integer input.
#include "fir_plain.cuh"
#include "fir_plain_tile.cuh"
#include "ptx.cuh"

#include <cuda_runtime.h>

namespace rfx {

static __device__ unsigned int g_fault_fir_plain;

namespace {

constexpr int kThreads = kPlainThreads;
constexpr int kTile = kPlainTileOutputs;

// One tile per block, the whole block as the tile's thread group.
template <int kFmt = 0>
__device__ __forceinline__ void plain_block_tile(const void* x, const float* taps, float2* y,
                                                 long long n, int num_taps, long long tile,
                                                 unsigned char* smem)
{
    uint32_t phase = 0;
    fir_plain_tile<kFmt>(x, taps, y, n, num_taps, tile, smem, &g_fault_fir_plain,
                         static_cast<int>(threadIdx.x), PlainBlockSync{}, phase, true);
}

}  // namespace

__global__ void __launch_bounds__(kThreads, 4)
fir_plain_kernel(const float2* __restrict__ x, const float* __restrict__ taps,
                 float2* __restrict__ y, long long n, int num_taps)
{
    extern __shared__ __align__(128) unsigned char smem[];
    plain_block_tile(x, taps, y, n, num_taps, blockIdx.x, smem);
}

// Several captures sharing one tap set: blockIdx.y picks the capture; blocks past a shorter
// capture's end return at once (as the project's batched kernels, src/fused.cu:141-162).
__global__ void __launch_bounds__(kThreads, 4)
fir_plain_batched_kernel(PlainBatch batch, const float* __restrict__ taps, int num_taps)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int c = blockIdx.y;
    const long long n = batch.num_samples[c];
    if (static_cast<long long>(blockIdx.x) * kTile >= n) {
        return;
    }
    plain_block_tile(batch.x[c], taps, static_cast<float2*>(batch.y[c]), n, num_taps, blockIdx.x,
                     smem);
}

// Captures with their own taps: block b takes tile b - tile0[c] of the capture c whose tiles
// contain it (same arithmetic per capture as fir_plain_kernel, so the same bits).
__global__ void __launch_bounds__(kThreads, 4)
fir_plain_caps_kernel(const __grid_constant__ PlainCaps caps)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const int block = static_cast<int>(blockIdx.x);
    int lo = 0;
    int hi = caps.count;
    while (hi - lo > 1) {
        const int mid = (lo + hi) / 2;
        if (caps.tile0[mid] <= block) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    plain_block_tile(caps.x[lo], caps.taps[lo], static_cast<float2*>(caps.y[lo]),
                     caps.num_samples[lo], caps.num_taps[lo], block - caps.tile0[lo], smem);
}

// Integer I/Q input (ci16, ci8), decoded in the load stage.
template <int kFmt>
__global__ void __launch_bounds__(kThreads, 4)
fir_plain_fmt_kernel(const void* __restrict__ x, const float* __restrict__ taps,
                     float2* __restrict__ y, long long n, int num_taps)
{
    extern __shared__ __align__(128) unsigned char smem[];
    plain_block_tile<kFmt>(x, taps, y, n, num_taps, blockIdx.x, smem);
}

size_t fir_plain_smem_bytes(int num_taps) { return plain_layout(num_taps).bytes; }

static cudaError_t ensure_smem_attr(const void* fn, size_t bytes)
{
    // The opt-in limit only has to be raised once per function and size class; raising it to
    // the device maximum once covers every tap count.
    if (bytes <= 48 * 1024) {
        return cudaSuccess;
    }
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) {
        return err;
    }
    int optin = 0;
    err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (err != cudaSuccess) {
        return err;
    }
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
}

cudaError_t fir_plain_launch(const void* x, const float* taps, void* y, long long n,
                             int num_taps, cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    const size_t bytes = fir_plain_smem_bytes(num_taps);
    cudaError_t err = ensure_smem_attr(reinterpret_cast<const void*>(fir_plain_kernel), bytes);
    if (err != cudaSuccess) {
        return err;
    }
    const long long tiles = (n + kTile - 1) / kTile;
    fir_plain_kernel<<<static_cast<unsigned>(tiles), kThreads, bytes, stream>>>(
        static_cast<const float2*>(x), taps, static_cast<float2*>(y), n, num_taps);
    return cudaGetLastError();
}

cudaError_t fir_plain_batched_launch(const PlainBatch& batch, int count, const float* taps,
                                     int num_taps, cudaStream_t stream)
{
    long long longest = 0;
    for (int c = 0; c < count; ++c) {
        longest = batch.num_samples[c] > longest ? batch.num_samples[c] : longest;
    }
    if (longest == 0) {
        return cudaSuccess;
    }
    const size_t bytes = fir_plain_smem_bytes(num_taps);
    cudaError_t err =
        ensure_smem_attr(reinterpret_cast<const void*>(fir_plain_batched_kernel), bytes);
    if (err != cudaSuccess) {
        return err;
    }
    const dim3 grid(static_cast<unsigned>((longest + kTile - 1) / kTile), count);
    fir_plain_batched_kernel<<<grid, kThreads, bytes, stream>>>(batch, taps, num_taps);
    return cudaGetLastError();
}

cudaError_t fir_plain_launch_format(int format, const void* x, const float* taps, void* y,
                                    long long n, int num_taps, cudaStream_t stream)
{
    if (format == 0) {
        return fir_plain_launch(x, taps, y, n, num_taps, stream);
    }
    if (n <= 0) {
        return cudaSuccess;
    }
    const size_t bytes = plain_layout(num_taps, format).bytes;
    const void* fn = format == 1 ? reinterpret_cast<const void*>(fir_plain_fmt_kernel<1>)
                                 : reinterpret_cast<const void*>(fir_plain_fmt_kernel<2>);
    cudaError_t err = ensure_smem_attr(fn, bytes);
    if (err != cudaSuccess) {
        return err;
    }
    const long long tiles = (n + kTile - 1) / kTile;
    if (format == 1) {
        fir_plain_fmt_kernel<1><<<static_cast<unsigned>(tiles), kThreads, bytes, stream>>>(
            x, taps, static_cast<float2*>(y), n, num_taps);
    } else {
        fir_plain_fmt_kernel<2><<<static_cast<unsigned>(tiles), kThreads, bytes, stream>>>(
            x, taps, static_cast<float2*>(y), n, num_taps);
    }
    return cudaGetLastError();
}

cudaError_t fir_plain_caps_launch(const PlainCaps& caps, cudaStream_t stream)
{
    const int tiles = caps.tile0[caps.count];
    if (caps.count == 0 || tiles == 0) {
        return cudaSuccess;
    }
    int kmax = 1;
    for (int c = 0; c < caps.count; ++c) {
        kmax = caps.num_taps[c] > kmax ? caps.num_taps[c] : kmax;
    }
    const size_t bytes = fir_plain_smem_bytes(kmax);
    cudaError_t err =
        ensure_smem_attr(reinterpret_cast<const void*>(fir_plain_caps_kernel), bytes);
    if (err != cudaSuccess) {
        return err;
    }
    fir_plain_caps_kernel<<<static_cast<unsigned>(tiles), kThreads, bytes, stream>>>(caps);
    return cudaGetLastError();
}

cudaError_t fir_plain_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_fir_plain, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_fir_plain, &zero, sizeof(unsigned int));
}

}  // namespace rfx
