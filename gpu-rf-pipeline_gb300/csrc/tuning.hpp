// The tuned-configuration tables consulted by RFX_FIR_AUTO, the tensor-core FIR launches and
// RFX_CHAN_AUTO plans (tuning.cu), filled by rfx_autotune_fir / rfx_autotune_channelize and
// persisted with rfx_autotune_save/load.
#pragma once

#include "fir_tc.cuh"

namespace rfx {

int tuned_fir_impl(int num_taps, long long n);
TcConfig tuned_fir_tc_config(int num_taps, long long n);
int tuned_chan_impl(int channels, long long n);
// log2 of the plain channelizer's chunk in samples (0: no chunks), tuned or the built-in 21.
int tuned_chan_chunk_log2(int channels, long long n);

}  // namespace rfx

struct rfx_chan_plan;
namespace rfx {
// rfx_chan_plan_create with the plain form's chunk size given (log2 of samples; 0: one pass;
// -1: the tuned or built-in size). Defined with the C ABI (rfx_api.cu).
int chan_plan_create_chunked(int impl, int channels, long long max_samples, int chunk_log2,
                             rfx_chan_plan** plan);

}  // namespace rfx
