// The tuned-configuration table consulted by RFX_FIR_AUTO and the tensor-core launches
// (tuning.cu), filled by rfx_autotune_fir and persisted with rfx_autotune_save/load.
#pragma once

#include "fir_tc.cuh"

namespace rfx {

int tuned_fir_impl(int num_taps, long long n);
TcConfig tuned_fir_tc_config(int num_taps, long long n);

}  // namespace rfx
