// Tensor-core FIR (fir_tc.cu) and the per-capture batch (fir_batch.cu): internal interface.
#pragma once

#include "rfx.h"

#include <cuda_runtime.h>

namespace rfx {

// Form and tile shape of the tensor-core FIR, chosen by the tuner.
struct TcConfig {
    int tile_blocks;  // 128-output blocks per tile: 96 = one CTA per tile (fir_tc.cu),
                      // 192 = a CTA pair per tile of 96 256-output blocks (fir_tc2.cu),
                      // 48 = the resident-window form, 2 to 1025 taps (fir_tc_win.cu)
    int stages;       // operand ring depth cap (the largest that fits is used)
};
constexpr int kTcPairTile = 192;
constexpr int kTcWindowTile = 48;

constexpr int kTcBatchMax = 4096;

// Whether the tensor-core kernel takes this tap count. One tap is an exact elementwise scale,
// which the plain kernel computes exactly; the split form would round it.
bool fir_tc_supported(int num_taps);

cudaError_t fir_tc_launch(const void* x, const float* taps, void* y, long long n, int num_taps,
                          TcConfig config, cudaStream_t stream);
cudaError_t fir_tc_take_fault(unsigned int* code);

// The resident-window form (fir_tc_win.cu): 2 to 1025 taps, tiles of 48 blocks whose whole input
// window arrives by one TMA copy; format 0 cf32, 1 ci16, 2 ci8 (decoded in the load stage, the
// same bits as over the converted samples). n >= 128.
bool fir_tcw_supported(int num_taps);
long long fir_tcw_tile_outputs();
cudaError_t fir_tcw_launch(int format, const void* x, const float* taps, void* y, long long n,
                           int num_taps, cudaStream_t stream);
cudaError_t fir_tcw_take_fault(unsigned int* code);

// The same FIR over integer I/Q input decoded in the load stage (format 1 = ci16, 2 = ci8; 0 =
// cf32, fir_tc_launch): the copies move the stored components, the producers convert them as
// the project's SigMF reader does. Results have the bits of fir_tc_launch over the converted
// samples in the single-CTA form (the form integer input always takes).
cudaError_t fir_tc_launch_format(int format, const void* x, const float* taps, void* y,
                                 long long n, int num_taps, TcConfig config, cudaStream_t stream);
long long fir_tc_tile_outputs_format(int format, int num_taps, long long n, TcConfig config);

// Outputs per tile of the form fir_tc_launch picks for (num_taps, n, config): tiles start at
// multiples of this, and each tile's results depend only on the samples from one tile before
// its start to its end (its window reaches back C blocks, C * 128 <= 3456 < one tile), so a
// run over any tile-aligned stretch with one tile of history reproduces the whole run's bits
// there. 1 when the plain kernel runs instead.
long long fir_tc_tile_outputs(int num_taps, long long n, TcConfig config);

// Per-capture-taps batch: tensor core (or auto) = one persistent launch of fir_batch.cu per
// 96 captures; plain = one launch per capture.
cudaError_t fir_batch_launch(int impl, const rfx_fir_capture* captures, int count,
                             cudaStream_t stream);
cudaError_t fir_batch_tc_launch(const rfx_fir_capture* captures, int count, cudaStream_t stream);
bool fir_batch_supported(int num_taps);

// A batch plan: the work list of one batch (capture tables, tensor maps, per-block ranges) in
// device memory, built once; every run is ONE persistent launch of fir_batch.cu that takes the
// tensor-core captures and, with groups of its threads, the plain captures' tiles.
struct BatchPlan;
cudaError_t fir_batch_plan_make(int impl, const rfx_fir_capture* captures, int count,
                                BatchPlan** out);
cudaError_t fir_batch_plan_run(const BatchPlan* plan, cudaStream_t stream);
void fir_batch_plan_free(BatchPlan* plan);
void fir_batch_plan_counts(const BatchPlan* plan, int* tc_captures, int* plain_captures,
                           int* launches);
cudaError_t fir_batch_take_fault(unsigned int* code);

}  // namespace rfx
