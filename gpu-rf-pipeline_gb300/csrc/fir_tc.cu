// Tensor-core FIR: placeholder until the tcgen05 kernel lands; every call reports
// cudaErrorNotSupported, and one-tap calls never reach here.
#include "fir_tc.cuh"
#include "fir_plain.cuh"

namespace rfx {

static __device__ unsigned int g_fault_fir_tc;

bool fir_tc_supported(int num_taps) { return num_taps > 1; }

cudaError_t fir_tc_launch(const void*, const float*, void*, long long, int, TcConfig,
                          cudaStream_t)
{
    return cudaErrorNotSupported;
}

cudaError_t fir_tc_take_fault(unsigned int* code)
{
    unsigned int zero = 0;
    cudaError_t err = cudaMemcpyFromSymbol(code, g_fault_fir_tc, sizeof(unsigned int));
    if (err != cudaSuccess) {
        return err;
    }
    return cudaMemcpyToSymbol(g_fault_fir_tc, &zero, sizeof(unsigned int));
}

cudaError_t fir_batch_launch(int impl, const rfx_fir_capture* captures, int count,
                             cudaStream_t stream)
{
    for (int c = 0; c < count; ++c) {
        if (captures[c].num_samples == 0) {
            continue;
        }
        cudaError_t err = (impl == RFX_FIR_TC && fir_tc_supported(captures[c].num_taps))
                              ? fir_tc_launch(captures[c].x, captures[c].taps, captures[c].y,
                                              captures[c].num_samples, captures[c].num_taps,
                                              TcConfig{128, 4}, stream)
                              : fir_plain_launch(captures[c].x, captures[c].taps, captures[c].y,
                                                 captures[c].num_samples, captures[c].num_taps,
                                                 stream);
        if (err != cudaSuccess) {
            return err;
        }
    }
    return cudaSuccess;
}

}  // namespace rfx
