// Plain FP32 FIR kernels (fir_plain.cu): internal launch interface used by the C ABI.
#pragma once

#include <cstddef>
#include <cuda_runtime.h>

namespace rfx {

constexpr int kPlainThreads = 256;
constexpr int kPlainOutputsPerThread = 9;
constexpr int kPlainTileOutputs = kPlainThreads * kPlainOutputsPerThread;  // 2304
constexpr int kMaxTaps = 8192;  // the project's constant-bank capacity (src/fir.cu:208)

// Captures sharing one tap set, passed by value as one kernel argument (64 * 24 bytes).
constexpr int kPlainBatchMax = 64;
struct PlainBatch {
    const void* x[kPlainBatchMax];
    void* y[kPlainBatchMax];
    long long num_samples[kPlainBatchMax];
};

// Captures with their own taps, one launch for all: blocks take the captures' tiles in order
// (tile0[c] = first block of capture c). Passed by value as one kernel argument.
constexpr int kPlainCapsMax = 256;
struct PlainCaps {
    const void* x[kPlainCapsMax];
    void* y[kPlainCapsMax];
    const float* taps[kPlainCapsMax];
    long long num_samples[kPlainCapsMax];
    int num_taps[kPlainCapsMax];
    int tile0[kPlainCapsMax + 1];
    int count;
};

size_t fir_plain_smem_bytes(int num_taps);
cudaError_t fir_plain_launch(const void* x, const float* taps, void* y, long long n,
                             int num_taps, cudaStream_t stream);
cudaError_t fir_plain_batched_launch(const PlainBatch& batch, int count, const float* taps,
                                     int num_taps, cudaStream_t stream);
// The FIR of integer I/Q input decoded in the load stage: format 1 = ci16 (components x / 32768),
// 2 = ci8 (x / 128), 0 = cf32 (fir_plain_launch). Same bits as decoding first.
cudaError_t fir_plain_launch_format(int format, const void* x, const float* taps, void* y,
                                    long long n, int num_taps, cudaStream_t stream);

// Up to kPlainCapsMax captures (non-empty), each with its own taps, in one launch.
cudaError_t fir_plain_caps_launch(const PlainCaps& caps, cudaStream_t stream);
cudaError_t fir_plain_take_fault(unsigned int* code);

}  // namespace rfx
