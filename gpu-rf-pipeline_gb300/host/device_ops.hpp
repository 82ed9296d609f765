#pragma once

// Device-pointer entry points with the project's names and signatures (src/device_ops.hpp),
// on top of the C ABI (include/rfx.h). Each one only enqueues work: no allocation, no host
// transfer, no synchronization. Errors throw std::runtime_error.

#include "rfx.h"
#include "types.hpp"

#include <cuda_runtime.h>
#include <cufft.h>

// The project's four variants keep their names and map to this library's plain FP32 kernel,
// which computes the same fused multiply-add chain, so their results are unchanged bit for bit.
// Plain, TcSplit and Auto are this library's own (include/rfx.h, rfx_fir_impl).
enum class FirImpl { Naive, Tiled, TiledConst, Register, Plain, TcSplit, Auto };

bool parse_fir_impl(const char* name, FirImpl& impl);
int to_rfx_impl(FirImpl impl);

void fir_device(FirImpl impl, const cf32* x, const float* taps, cf32* y, int num_samples,
                int num_taps);
void fir_load_const_taps(const float* taps, int num_taps, cudaStream_t stream);
void fir_launch(FirImpl impl, const cf32* x, const float* taps, cf32* y, int num_samples,
                int num_taps, cudaStream_t stream);
void fir_naive_device(const cf32* x, const float* taps, cf32* y, int num_samples, int num_taps);

// The project caps a shared-taps batch at kMaxFirBatch channels (its fusion group size); this
// library takes any count, so generated code that respects the cap keeps working.
constexpr int kMaxFirBatch = 8;
void fir_batched_device(FirImpl impl, const cf32* const* x, cf32* const* y,
                        const int* num_samples, int count, const float* taps, int num_taps);
void fir_naive_batched_device(const cf32* const* x, cf32* const* y, const int* num_samples,
                              int count, const float* taps, int num_taps);

// mag[n] = |x[n]| for n < num_samples, on the legacy default stream (src/device_ops.hpp:57).
void magnitude_device(const cf32* x, float* mag, int num_samples);

int channelize_frames(int num_samples, int channels);

// The project's signature: branch sums into `out`, then `plan` (a batched FftPlan of `channels`
// points times channelize_frames() frames) run as an inverse transform in place.
void channelize_device(cufftHandle plan, const cf32* x, const float* taps, cf32* out,
                       int num_samples, int channels, int num_taps);

// Any implementation through an rfx_chan_plan (rfx_chan_plan_create).
void channelize_device(rfx_chan_plan* plan, const cf32* x, const float* taps, cf32* out,
                       int num_samples, int num_taps, cudaStream_t stream = nullptr);

// channelize |> magnitude through a plan: mag is frames x channels floats.
void channelize_magnitude_device(rfx_chan_plan* plan, const cf32* x, const float* taps,
                                 float* mag, int num_samples, int num_taps,
                                 cudaStream_t stream = nullptr);
