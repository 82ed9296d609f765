// The tuned-configuration tables consulted by RFX_FIR_AUTO, the tensor-core FIR launches and
// RFX_CHAN_AUTO plans (tuning.cu), filled by rfx_autotune_fir / rfx_autotune_channelize and
// persisted with rfx_autotune_save/load.
#pragma once

#include "fir_tc.cuh"

namespace rfx {

int tuned_fir_impl(int num_taps, long long n);
int tuned_fir_batch_impl(int num_taps, long long n);
int tuned_fir_batch_launch_impl(int num_taps, long long n);
TcConfig tuned_fir_tc_config(int num_taps, long long n);
int tuned_chan_impl(int channels, long long n);

}  // namespace rfx
