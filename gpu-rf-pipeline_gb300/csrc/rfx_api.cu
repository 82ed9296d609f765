// The C ABI of librfx.so (include/rfx.h): argument checks, implementation dispatch, channelizer
// plans, host-buffer operations with phase timing, and the fault word readout.
#include "rfx.h"

#include "api_error.hpp"

#include "chan_plain.cuh"
#include "chan_tc.cuh"
#include "chan_wide.cuh"
#include "fir_plain.cuh"
#include "fir_tc.cuh"
#include "fir_tc2.cuh"
#include "magnitude.cuh"
#include "tuning.hpp"

#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int cuda_fail(cudaError_t err, const char* what)
{
    return fail(RFX_ERR_CUDA, "CUDA error: %s (code %d) in %s", cudaGetErrorString(err),
                static_cast<int>(err), what);
}

const char* cufft_text(cufftResult r)
{
    switch (r) {
    case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
    case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
    case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
    case CUFFT_INVALID_TYPE: return "CUFFT_INVALID_TYPE";
    case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
    case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
    case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
    case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
    case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
    case CUFFT_UNALIGNED_DATA: return "CUFFT_UNALIGNED_DATA";
    default: return "cuFFT error";
    }
}

int cufft_fail(cufftResult r, const char* what)
{
    return fail(RFX_ERR_CUDA, "cuFFT error: %s (code %d) in %s", cufft_text(r),
                static_cast<int>(r), what);
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

constexpr int64_t kMaxSamples = INT32_MAX;

const char* const kFirImplNames[] = {"plain", "tc_split", "auto"};
const char* const kChanImplNames[] = {"plain", "tc_split", "auto"};

int check_fir_args(int impl, const void* x, const float* taps, const void* y, int64_t n,
                   int num_taps)
{
    if (impl < RFX_FIR_PLAIN || impl > RFX_FIR_AUTO) {
        return fail(RFX_ERR_INVALID, "fir: unknown implementation %d", impl);
    }
    if (n < 0 || n > kMaxSamples) {
        return fail(RFX_ERR_INVALID, "fir: %lld samples, expected 0 to %lld",
                    static_cast<long long>(n), static_cast<long long>(kMaxSamples));
    }
    if (num_taps < 1) {
        return fail(RFX_ERR_INVALID, "fir: need at least one tap");
    }
    if (num_taps > rfx::kMaxTaps) {
        return fail(RFX_ERR_CAPACITY, "fir: %d taps, more than the %d supported", num_taps,
                    rfx::kMaxTaps);
    }
    if (n > 0 && (x == nullptr || y == nullptr || taps == nullptr)) {
        return fail(RFX_ERR_INVALID, "fir: null pointer");
    }
    if (n > 0 && (!aligned16(x) || !aligned16(y))) {
        return fail(RFX_ERR_ALIGNMENT, "fir: sample buffers must be 16-byte aligned");
    }
    if (n > 0 && (reinterpret_cast<uintptr_t>(taps) & 3u) != 0) {
        return fail(RFX_ERR_ALIGNMENT, "fir: taps must be 4-byte aligned");
    }
    return RFX_OK;
}

// Resolves RFX_FIR_AUTO and the cases the tensor-core kernel hands to the plain one.
int resolve_fir_impl(int impl, int num_taps, int64_t n)
{
    if (impl == RFX_FIR_AUTO) {
        impl = rfx::tuned_fir_impl(num_taps, n);
    }
    if (impl == RFX_FIR_TC && !rfx::fir_tc_supported(num_taps)) {
        impl = RFX_FIR_PLAIN;  // one tap: an exact elementwise scale, see fir_tc_supported
    }
    return impl;
}

size_t format_sample_bytes(int format) { return format == RFX_FORMAT_CF32 ? 8 : format == RFX_FORMAT_CI16 ? 4 : 2; }

int check_format(int format)
{
    if (format < RFX_FORMAT_CF32 || format > RFX_FORMAT_CI8) {
        return fail(RFX_ERR_INVALID, "fir: unknown sample format %d", format);
    }
    return RFX_OK;
}

int launch_fir_format(int impl, int format, const void* x, const float* taps, void* y, int64_t n,
                      int num_taps, cudaStream_t stream)
{
    cudaError_t err;
    if (impl == RFX_FIR_TC) {
        err = rfx::fir_tc_launch_format(format, x, taps, y, n, num_taps,
                                        rfx::tuned_fir_tc_config(num_taps, n), stream);
        return err == cudaSuccess ? RFX_OK : cuda_fail(err, "fir_tc_launch_format");
    }
    err = rfx::fir_plain_launch_format(format, x, taps, y, n, num_taps, stream);
    return err == cudaSuccess ? RFX_OK : cuda_fail(err, "fir_plain_launch_format");
}

int launch_fir(int impl, const void* x, const float* taps, void* y, int64_t n, int num_taps,
               cudaStream_t stream)
{
    cudaError_t err;
    if (impl == RFX_FIR_TC) {
        err = rfx::fir_tc_launch(x, taps, y, n, num_taps, rfx::tuned_fir_tc_config(num_taps, n),
                                 stream);
        return err == cudaSuccess ? RFX_OK : cuda_fail(err, "fir_tc_launch");
    }
    err = rfx::fir_plain_launch(x, taps, y, n, num_taps, stream);
    return err == cudaSuccess ? RFX_OK : cuda_fail(err, "fir_plain_launch");
}

}  // namespace

namespace rfx {

int set_last_error(int status, const char* message) { return fail(status, "%s", message); }

}  // namespace rfx

struct rfx_chan_plan;
namespace {
int channelize_plan(rfx_chan_plan* plan, const void* x, const float* taps, void* out,
                    int64_t num_samples, int num_taps, cudaStream_t stream, bool magnitude,
                    int format);
}  // namespace

struct rfx_chan_plan {
    int impl;
    int channels;
    int64_t frames;       // cuFFT batch (plain); maximum frames (tensor core)
    cufftHandle fft;
    bool has_fft;
    void* twiddles;       // tensor core: the DFT operand image, built once in FP64
    void* scratch;        // plain: channel outputs before their magnitude (first such call);
                          // tensor core, 1024 channels: the branch sums (made with the plan)
};

extern "C" {

const char* rfx_last_error(void) { return g_last_error.c_str(); }

const char* rfx_version(void) { return "rfx 0.1.0 sm_103a"; }

int rfx_device_fault(unsigned int* code)
{
    if (code == nullptr) {
        return fail(RFX_ERR_INVALID, "rfx_device_fault: null pointer");
    }
    cudaError_t err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        return cuda_fail(err, "cudaDeviceSynchronize");
    }
    unsigned int total = 0;
    unsigned int part = 0;
    if ((err = rfx::fir_plain_take_fault(&part)) != cudaSuccess) {
        return cuda_fail(err, "fir_plain fault word");
    }
    total |= part;
    part = 0;
    if ((err = rfx::fir_tc_take_fault(&part)) != cudaSuccess) {
        return cuda_fail(err, "fir_tc fault word");
    }
    total |= part;
    part = 0;
    if ((err = rfx::fir_tcw_take_fault(&part)) != cudaSuccess) {
        return cuda_fail(err, "fir_tcw fault word");
    }
    total |= part;
    part = 0;
    if ((err = rfx::fir_tc2_take_fault(&part)) != cudaSuccess) {
        return cuda_fail(err, "fir_tc2 fault word");
    }
    total |= part;
    part = 0;
    if ((err = rfx::fir_batch_take_fault(&part)) != cudaSuccess) {
        return cuda_fail(err, "fir_batch fault word");
    }
    total |= part;
    part = 0;
    if ((err = rfx::chan_tc_take_fault(&part)) != cudaSuccess) {
        return cuda_fail(err, "chan_tc fault word");
    }
    total |= part;
    part = 0;
    if ((err = rfx::chan_wide_take_fault(&part)) != cudaSuccess) {
        return cuda_fail(err, "chan_wide fault word");
    }
    total |= part;
    *code = total;
    return RFX_OK;
}

int rfx_fir_impl_name(int index, char* name, size_t size)
{
    if (index < 0 || index >= 3 || name == nullptr || size == 0) {
        return RFX_ERR_INVALID;
    }
    std::snprintf(name, size, "%s", kFirImplNames[index]);
    return RFX_OK;
}

int rfx_chan_impl_name(int index, char* name, size_t size)
{
    if (index < 0 || index >= 3 || name == nullptr || size == 0) {
        return RFX_ERR_INVALID;
    }
    std::snprintf(name, size, "%s", kChanImplNames[index]);
    return RFX_OK;
}

int rfx_parse_fir_impl(const char* name, int* impl)
{
    if (name == nullptr || impl == nullptr) {
        return fail(RFX_ERR_INVALID, "rfx_parse_fir_impl: null pointer");
    }
    static const struct {
        const char* name;
        int impl;
    } table[] = {{"plain", RFX_FIR_PLAIN}, {"tc_split", RFX_FIR_TC}, {"auto", RFX_FIR_AUTO},
                 {"naive", RFX_FIR_PLAIN}, {"tiled", RFX_FIR_PLAIN},
                 {"tiled_const", RFX_FIR_PLAIN}, {"register", RFX_FIR_PLAIN}};
    for (const auto& row : table) {
        if (std::strcmp(name, row.name) == 0) {
            *impl = row.impl;
            return RFX_OK;
        }
    }
    return fail(RFX_ERR_INVALID, "unknown fir implementation '%s'", name);
}

int rfx_parse_chan_impl(const char* name, int* impl)
{
    if (name == nullptr || impl == nullptr) {
        return fail(RFX_ERR_INVALID, "rfx_parse_chan_impl: null pointer");
    }
    for (int i = 0; i < 3; ++i) {
        if (std::strcmp(name, kChanImplNames[i]) == 0) {
            *impl = i;
            return RFX_OK;
        }
    }
    if (std::strcmp(name, "polyphase") == 0) {  // the project's report name for its one impl
        *impl = RFX_CHAN_PLAIN;
        return RFX_OK;
    }
    return fail(RFX_ERR_INVALID, "unknown channelize implementation '%s'", name);
}

// ---- FIR ---------------------------------------------------------------------------------

int rfx_fir_launch(int impl, const void* x, const float* taps, void* y, int64_t num_samples,
                   int num_taps, cudaStream_t stream)
{
    const int rc = check_fir_args(impl, x, taps, y, num_samples, num_taps);
    if (rc != RFX_OK || num_samples == 0) {
        return rc;
    }
    return launch_fir(resolve_fir_impl(impl, num_taps, num_samples), x, taps, y, num_samples,
                      num_taps, stream);
}

int rfx_fir_launch_format(int impl, int format, const void* x, const float* taps, void* y,
                          int64_t num_samples, int num_taps, cudaStream_t stream)
{
    int rc = check_format(format);
    if (rc == RFX_OK) {
        rc = check_fir_args(impl, x, taps, y, num_samples, num_taps);
    }
    if (rc != RFX_OK || num_samples == 0) {
        return rc;
    }
    return launch_fir_format(resolve_fir_impl(impl, num_taps, num_samples), format, x, taps, y,
                             num_samples, num_taps, stream);
}

int rfx_fir_impl_used(int impl, int num_taps, int64_t num_samples, int batch, int* used)
{
    if (used == nullptr) {
        return fail(RFX_ERR_INVALID, "fir_impl_used: null result pointer");
    }
    if (impl < RFX_FIR_PLAIN || impl > RFX_FIR_AUTO) {
        return fail(RFX_ERR_INVALID, "fir_impl_used: unknown implementation %d", impl);
    }
    if (num_taps < 1 || num_taps > rfx::kMaxTaps || num_samples < 0) {
        return fail(RFX_ERR_INVALID, "fir_impl_used: %d taps, %lld samples", num_taps,
                    static_cast<long long>(num_samples));
    }
    int r = impl == RFX_FIR_AUTO && batch != 0
                ? resolve_fir_impl(rfx::tuned_fir_batch_impl(num_taps, num_samples), num_taps,
                                   num_samples)
                : resolve_fir_impl(impl, num_taps, num_samples);
    constexpr int64_t kBlockOutputs = 128;  // the tensor-core kernels' output block
    if (r == RFX_FIR_TC && num_samples < kBlockOutputs) {
        r = RFX_FIR_PLAIN;  // no whole block to compute: the plain kernel is exact
    }
    if (r == RFX_FIR_TC && batch != 0 && !rfx::fir_batch_supported(num_taps)) {
        r = RFX_FIR_PLAIN;  // the persistent batch kernel's shared-memory budget is smaller
    }
    *used = r;
    return RFX_OK;
}

int rfx_fir_device(int impl, const void* x, const float* taps, void* y, int64_t num_samples,
                   int num_taps)
{
    return rfx_fir_launch(impl, x, taps, y, num_samples, num_taps, nullptr);
}

int rfx_fir_load_const_taps(const float* taps, int num_taps, cudaStream_t stream)
{
    (void)stream;
    if (num_taps < 1) {
        return fail(RFX_ERR_INVALID, "fir: need at least one tap");
    }
    if (num_taps > rfx::kMaxTaps) {
        return fail(RFX_ERR_CAPACITY, "fir: %d taps, more than the %d supported", num_taps,
                    rfx::kMaxTaps);
    }
    if (taps == nullptr) {
        return fail(RFX_ERR_INVALID, "fir: null taps");
    }
    return RFX_OK;
}

int rfx_fir_batched_device(int impl, const void* const* x, void* const* y,
                           const int64_t* num_samples, int count, const float* taps,
                           int num_taps, cudaStream_t stream)
{
    if (count < 1 || x == nullptr || y == nullptr || num_samples == nullptr) {
        return fail(RFX_ERR_INVALID, "batched fir: %d channels, expected at least 1", count);
    }
    int64_t longest = 0;
    for (int c = 0; c < count; ++c) {
        const int rc = check_fir_args(impl, x[c], taps, y[c], num_samples[c], num_taps);
        if (rc != RFX_OK) {
            return rc;
        }
        longest = std::max(longest, num_samples[c]);
    }
    const int resolved = resolve_fir_impl(impl, num_taps, longest);
    if (resolved == RFX_FIR_TC) {
        for (int c = 0; c < count; ++c) {
            if (num_samples[c] == 0) {
                continue;
            }
            const int rc = launch_fir(resolved, x[c], taps, y[c], num_samples[c], num_taps,
                                      stream);
            if (rc != RFX_OK) {
                return rc;
            }
        }
        return RFX_OK;
    }
    for (int first = 0; first < count; first += rfx::kPlainBatchMax) {
        const int chunk = std::min(count - first, rfx::kPlainBatchMax);
        rfx::PlainBatch batch{};
        for (int c = 0; c < chunk; ++c) {
            batch.x[c] = x[first + c];
            batch.y[c] = y[first + c];
            batch.num_samples[c] = num_samples[first + c];
        }
        const cudaError_t err =
            rfx::fir_plain_batched_launch(batch, chunk, taps, num_taps, stream);
        if (err != cudaSuccess) {
            return cuda_fail(err, "fir_plain_batched_launch");
        }
    }
    return RFX_OK;
}

int rfx_fir_batch_launch(int impl, const rfx_fir_capture* captures, int count,
                         cudaStream_t stream)
{
    if (count < 1 || count > rfx::kTcBatchMax || captures == nullptr) {
        return fail(RFX_ERR_INVALID, "fir batch: %d captures, expected 1 to %d", count,
                    rfx::kTcBatchMax);
    }
    for (int c = 0; c < count; ++c) {
        const rfx_fir_capture& cap = captures[c];
        const int rc = check_fir_args(impl, cap.x, cap.taps, cap.y, cap.num_samples,
                                      cap.num_taps);
        if (rc != RFX_OK) {
            return rc;
        }
        if (cap.reserved != 0) {
            return fail(RFX_ERR_INVALID, "fir batch: capture %d: reserved field must be 0", c);
        }
    }
    cudaError_t err = rfx::fir_batch_launch(impl, captures, count, stream);
    return err == cudaSuccess ? RFX_OK : cuda_fail(err, "fir_batch_launch");
}

struct rfx_fir_batch_plan {
    rfx::BatchPlan* plan;
};

int rfx_fir_batch_plan_create(int impl, const rfx_fir_capture* captures, int count,
                              rfx_fir_batch_plan** plan)
{
    if (plan == nullptr) {
        return fail(RFX_ERR_INVALID, "fir batch plan: null plan pointer");
    }
    *plan = nullptr;
    if (count < 1 || count > rfx::kTcBatchMax || captures == nullptr) {
        return fail(RFX_ERR_INVALID, "fir batch plan: %d captures, expected 1 to %d", count,
                    rfx::kTcBatchMax);
    }
    for (int c = 0; c < count; ++c) {
        const rfx_fir_capture& cap = captures[c];
        const int rc = check_fir_args(impl, cap.x, cap.taps, cap.y, cap.num_samples,
                                      cap.num_taps);
        if (rc != RFX_OK) {
            return rc;
        }
        if (cap.reserved != 0) {
            return fail(RFX_ERR_INVALID, "fir batch plan: capture %d: reserved field must be 0",
                        c);
        }
    }
    rfx::BatchPlan* p = nullptr;
    const cudaError_t err = rfx::fir_batch_plan_make(impl, captures, count, &p);
    if (err != cudaSuccess) {
        return cuda_fail(err, "fir_batch_plan_make");
    }
    *plan = new rfx_fir_batch_plan{p};
    return RFX_OK;
}

int rfx_fir_batch_run(rfx_fir_batch_plan* plan, cudaStream_t stream)
{
    if (plan == nullptr) {
        return fail(RFX_ERR_INVALID, "fir batch run: null plan");
    }
    const cudaError_t err = rfx::fir_batch_plan_run(plan->plan, stream);
    return err == cudaSuccess ? RFX_OK : cuda_fail(err, "fir_batch_plan_run");
}

int rfx_fir_batch_plan_info(const rfx_fir_batch_plan* plan, int* tc_captures,
                            int* plain_captures, int* launches)
{
    if (plan == nullptr || tc_captures == nullptr || plain_captures == nullptr ||
        launches == nullptr) {
        return fail(RFX_ERR_INVALID, "fir batch plan info: null pointer");
    }
    rfx::fir_batch_plan_counts(plan->plan, tc_captures, plain_captures, launches);
    return RFX_OK;
}

int rfx_fir_batch_plan_destroy(rfx_fir_batch_plan* plan)
{
    if (plan != nullptr) {
        rfx::fir_batch_plan_free(plan->plan);
        delete plan;
    }
    return RFX_OK;
}

// ---- channelizer --------------------------------------------------------------------------

int64_t rfx_channelize_frames(int64_t num_samples, int channels)
{
    if (channels < 1 || num_samples < 0) {
        return 0;
    }
    return (num_samples + channels - 1) / channels;
}

int rfx_chan_plan_create(int impl, int channels, int64_t max_samples, rfx_chan_plan** plan)
{
    if (plan == nullptr) {
        return fail(RFX_ERR_INVALID, "channelize: null plan pointer");
    }
    *plan = nullptr;
    if (impl == RFX_CHAN_AUTO) {
        impl = rfx::tuned_chan_impl(channels, max_samples);
    }
    if (impl != RFX_CHAN_PLAIN && impl != RFX_CHAN_TC) {
        return fail(RFX_ERR_INVALID, "channelize: unknown implementation %d", impl);
    }
    if (channels < 1) {
        return fail(RFX_ERR_INVALID, "channelize: need at least one channel");
    }
    if (max_samples < 0 || max_samples > kMaxSamples) {
        return fail(RFX_ERR_INVALID, "channelize: %lld samples, expected 0 to %lld",
                    static_cast<long long>(max_samples), static_cast<long long>(kMaxSamples));
    }
    auto* p = new rfx_chan_plan{impl, channels, rfx_channelize_frames(max_samples, channels), 0,
                                false, nullptr, nullptr};
    if (impl == RFX_CHAN_TC) {
        const bool wide = rfx::chan_wide_supported(channels);
        if (!wide && !rfx::chan_tc_supported(channels, 1)) {
            delete p;
            return fail(RFX_ERR_CAPACITY, "channelize: the tensor-core form takes 64 or 1024 "
                                          "channels, not %d",
                        channels);
        }
        cudaError_t err = cudaMalloc(&p->twiddles, wide ? rfx::chan_wide_image_bytes()
                                                        : rfx::chan_tc_twiddle_bytes());
        if (err == cudaSuccess) {
            err = wide ? rfx::chan_wide_build_image(p->twiddles, nullptr)
                       : rfx::chan_tc_build_twiddles(p->twiddles, nullptr);
        }
        if (err == cudaSuccess && wide && p->frames > 0) {
            // The branch sums between the two kernels of the 1024-channel form.
            err = cudaMalloc(&p->scratch, static_cast<size_t>(p->frames) * channels * 8u);
            if (err != cudaSuccess) {
                p->scratch = nullptr;
            }
        }
        if (err == cudaSuccess) {
            err = cudaDeviceSynchronize();
        }
        if (err != cudaSuccess) {
            cudaFree(p->twiddles);
            cudaFree(p->scratch);
            delete p;
            return cuda_fail(err, "channelizer twiddles");
        }
        *plan = p;
        return RFX_OK;
    }
    if (p->frames > 0) {
        int nfft = channels;
        const cufftResult r = cufftPlanMany(&p->fft, 1, &nfft, nullptr, 1, nfft, nullptr, 1,
                                            nfft, CUFFT_C2C, static_cast<int>(p->frames));
        if (r != CUFFT_SUCCESS) {
            delete p;
            return cufft_fail(r, "cufftPlanMany");
        }
        p->has_fft = true;
    }
    *plan = p;
    return RFX_OK;
}

int rfx_chan_plan_destroy(rfx_chan_plan* plan)
{
    if (plan == nullptr) {
        return RFX_OK;
    }
    cufftResult r = CUFFT_SUCCESS;
    if (plan->has_fft) {
        r = cufftDestroy(plan->fft);
    }
    if (plan->twiddles != nullptr) {
        cudaFree(plan->twiddles);
    }
    if (plan->scratch != nullptr) {
        cudaFree(plan->scratch);
    }
    delete plan;
    return r == CUFFT_SUCCESS ? RFX_OK : cufft_fail(r, "cufftDestroy");
}

int rfx_channelize_launch(rfx_chan_plan* plan, const void* x, const float* taps, void* out,
                          int64_t num_samples, int num_taps, cudaStream_t stream)
{
    return channelize_plan(plan, x, taps, out, num_samples, num_taps, stream, false,
                           RFX_FORMAT_CF32);
}

int rfx_channelize_launch_format(rfx_chan_plan* plan, int format, int output, const void* x,
                                 const float* taps, void* out, int64_t num_samples, int num_taps,
                                 cudaStream_t stream)
{
    if (check_format(format) != RFX_OK) {
        return RFX_ERR_INVALID;
    }
    if (output != RFX_CHAN_OUT_COMPLEX && output != RFX_CHAN_OUT_MAGNITUDE) {
        return fail(RFX_ERR_INVALID, "channelize: unknown output %d", output);
    }
    return channelize_plan(plan, x, taps, out, num_samples, num_taps, stream,
                           output == RFX_CHAN_OUT_MAGNITUDE, format);
}

int rfx_channelize_magnitude_launch(rfx_chan_plan* plan, const void* x, const float* taps,
                                    float* mag, int64_t num_samples, int num_taps,
                                    cudaStream_t stream)
{
    return channelize_plan(plan, x, taps, mag, num_samples, num_taps, stream, true,
                           RFX_FORMAT_CF32);
}

int rfx_magnitude_launch(const void* x, float* mag, int64_t num_samples, cudaStream_t stream)
{
    if (num_samples < 0 || num_samples > kMaxSamples) {
        return fail(RFX_ERR_INVALID, "magnitude: %lld samples, expected 0 to %lld",
                    static_cast<long long>(num_samples), static_cast<long long>(kMaxSamples));
    }
    if (num_samples == 0) {
        return RFX_OK;
    }
    if (x == nullptr || mag == nullptr) {
        return fail(RFX_ERR_INVALID, "magnitude: null pointer");
    }
    if (!aligned16(x) || !aligned16(mag)) {
        return fail(RFX_ERR_ALIGNMENT, "magnitude: buffers must be 16-byte aligned");
    }
    const cudaError_t err = rfx::magnitude_launch(x, mag, num_samples, stream);
    return err == cudaSuccess ? RFX_OK : cuda_fail(err, "magnitude_launch");
}

}  // extern "C"

namespace {

// The channelizer through a plan; with `magnitude`, `out` receives |z| (float per channel):
// the tensor-core form computes it in its epilogue, the plain form runs the magnitude kernel
// over the channel outputs in the plan's scratch buffer (allocated by the first such call).
int channelize_plan(rfx_chan_plan* plan, const void* x, const float* taps, void* out,
                    int64_t num_samples, int num_taps, cudaStream_t stream, bool magnitude,
                    int format)
{
    if (plan == nullptr) {
        return fail(RFX_ERR_INVALID, "channelize: null plan");
    }
    if (num_samples < 0 || num_samples > kMaxSamples) {
        return fail(RFX_ERR_INVALID, "channelize: bad sample count %lld",
                    static_cast<long long>(num_samples));
    }
    if (num_taps < 1) {
        return fail(RFX_ERR_INVALID, "channelize: need at least one tap");
    }
    const int64_t frames = rfx_channelize_frames(num_samples, plan->channels);
    if (frames == 0) {
        return RFX_OK;
    }
    if (x == nullptr || taps == nullptr || out == nullptr) {
        return fail(RFX_ERR_INVALID, "channelize: null pointer");
    }
    if (!aligned16(x) || !aligned16(out)) {
        return fail(RFX_ERR_ALIGNMENT, "channelize: sample buffers must be 16-byte aligned");
    }
    if (plan->impl == RFX_CHAN_TC) {
        if (frames > plan->frames) {
            return fail(RFX_ERR_INVALID, "channelize: plan made for up to %lld frames, call has "
                                         "%lld",
                        static_cast<long long>(plan->frames), static_cast<long long>(frames));
        }
        if (rfx::chan_wide_supported(plan->channels)) {
            const cudaError_t err = rfx::chan_wide_launch(x, taps, plan->twiddles, plan->scratch,
                                                          out, num_samples, num_taps, stream,
                                                          magnitude, format);
            return err == cudaSuccess ? RFX_OK : cuda_fail(err, "chan_wide_launch");
        }
        if (!rfx::chan_tc_supported(plan->channels, num_taps)) {
            return fail(RFX_ERR_CAPACITY, "channelize: %d taps exceed the tensor-core form's "
                                          "shared memory",
                        num_taps);
        }
        const cudaError_t err = rfx::chan_tc_launch(x, taps, plan->twiddles, out, num_samples,
                                                    num_taps, stream, magnitude, format);
        return err == cudaSuccess ? RFX_OK : cuda_fail(err, "chan_tc_launch");
    }
    if (frames != plan->frames) {
        return fail(RFX_ERR_INVALID, "channelize: plan made for %lld frames, call has %lld",
                    static_cast<long long>(plan->frames), static_cast<long long>(frames));
    }
    void* z = out;
    if (magnitude) {
        if (plan->scratch == nullptr) {
            const cudaError_t e = cudaMalloc(&plan->scratch, static_cast<size_t>(plan->frames) *
                                                                 plan->channels * 8u);
            if (e != cudaSuccess) {
                plan->scratch = nullptr;
                return cuda_fail(e, "cudaMalloc (channelizer scratch)");
            }
        }
        z = plan->scratch;
    }
    cudaError_t err = rfx::chan_branch_launch(x, taps, z, frames, plan->channels, num_taps,
                                              stream, format);
    if (err != cudaSuccess) {
        return cuda_fail(err, "chan_branch_launch");
    }
    cufftResult r = cufftSetStream(plan->fft, stream);
    if (r != CUFFT_SUCCESS) {
        return cufft_fail(r, "cufftSetStream");
    }
    r = cufftExecC2C(plan->fft, static_cast<cufftComplex*>(z), static_cast<cufftComplex*>(z),
                     CUFFT_INVERSE);
    if (r != CUFFT_SUCCESS) {
        return cufft_fail(r, "cufftExecC2C");
    }
    if (magnitude) {
        err = rfx::magnitude_launch(z, static_cast<float*>(out), frames * plan->channels, stream);
        return err == cudaSuccess ? RFX_OK : cuda_fail(err, "magnitude_launch");
    }
    return RFX_OK;
}

}  // namespace

extern "C" {

int rfx_channelize_branches(const void* x, const float* taps, void* u, int64_t num_samples,
                            int channels, int num_taps, cudaStream_t stream)
{
    if (channels < 1 || num_taps < 1) {
        return fail(RFX_ERR_INVALID, "channelize: need at least one channel and one tap");
    }
    if (num_samples < 0 || num_samples > kMaxSamples) {
        return fail(RFX_ERR_INVALID, "channelize: bad sample count %lld",
                    static_cast<long long>(num_samples));
    }
    const int64_t frames = rfx_channelize_frames(num_samples, channels);
    if (frames == 0) {
        return RFX_OK;
    }
    if (x == nullptr || taps == nullptr || u == nullptr) {
        return fail(RFX_ERR_INVALID, "channelize: null pointer");
    }
    if (!aligned16(x) || !aligned16(u)) {
        return fail(RFX_ERR_ALIGNMENT, "channelize: sample buffers must be 16-byte aligned");
    }
    const cudaError_t err = rfx::chan_branch_launch(x, taps, u, frames, channels, num_taps,
                                                    stream);
    return err == cudaSuccess ? RFX_OK : cuda_fail(err, "chan_branch_launch");
}

// ---- host-buffer operations ----------------------------------------------------------------

}  // extern "C"

namespace {

struct DeviceMem {
    void* p = nullptr;
    ~DeviceMem()
    {
        if (p != nullptr) {
            cudaFree(p);
        }
    }
};

struct Event {
    cudaEvent_t e = nullptr;
    ~Event()
    {
        if (e != nullptr) {
            cudaEventDestroy(e);
        }
    }
};

void summarize(const std::vector<double>& v, double* mean, double* std_dev)
{
    *mean = 0.0;
    *std_dev = 0.0;
    if (v.empty()) {
        return;
    }
    double s = 0.0;
    for (double d : v) {
        s += d;
    }
    *mean = s / static_cast<double>(v.size());
    if (v.size() > 1) {
        double q = 0.0;
        for (double d : v) {
            q += (d - *mean) * (d - *mean);
        }
        *std_dev = std::sqrt(q / static_cast<double>(v.size() - 1));
    }
}

// warmup untimed passes, then `runs` passes with events around upload / compute / download on
// the legacy default stream (src/bench.cpp:65-93).
template <class Up, class Compute, class Down>
int timed_passes(rfx_bench* bench, Up up, Compute compute, Down down)
{
    const int warmup = bench != nullptr ? std::max(0, bench->warmup) : 0;
    const int runs = bench != nullptr ? std::max(1, bench->runs) : 1;
    for (int i = 0; i < warmup; ++i) {
        int rc;
        if ((rc = up()) != RFX_OK || (rc = compute()) != RFX_OK || (rc = down()) != RFX_OK) {
            return rc;
        }
    }
    Event start, uploaded, computed, downloaded;
    cudaError_t err;
    if ((err = cudaEventCreate(&start.e)) != cudaSuccess ||
        (err = cudaEventCreate(&uploaded.e)) != cudaSuccess ||
        (err = cudaEventCreate(&computed.e)) != cudaSuccess ||
        (err = cudaEventCreate(&downloaded.e)) != cudaSuccess) {
        return cuda_fail(err, "cudaEventCreate");
    }
    std::vector<double> h2d, kernel, d2h;
    for (int i = 0; i < runs; ++i) {
        int rc;
        cudaEventRecord(start.e, nullptr);
        if ((rc = up()) != RFX_OK) {
            return rc;
        }
        cudaEventRecord(uploaded.e, nullptr);
        if ((rc = compute()) != RFX_OK) {
            return rc;
        }
        cudaEventRecord(computed.e, nullptr);
        if ((rc = down()) != RFX_OK) {
            return rc;
        }
        cudaEventRecord(downloaded.e, nullptr);
        if ((err = cudaEventSynchronize(downloaded.e)) != cudaSuccess) {
            return cuda_fail(err, "cudaEventSynchronize");
        }
        float a = 0, b = 0, c = 0;
        cudaEventElapsedTime(&a, start.e, uploaded.e);
        cudaEventElapsedTime(&b, uploaded.e, computed.e);
        cudaEventElapsedTime(&c, computed.e, downloaded.e);
        h2d.push_back(a);
        kernel.push_back(b);
        d2h.push_back(c);
    }
    if (bench != nullptr) {
        summarize(h2d, &bench->h2d_ms_mean, &bench->h2d_ms_std);
        summarize(kernel, &bench->kernel_ms_mean, &bench->kernel_ms_std);
        summarize(d2h, &bench->d2h_ms_mean, &bench->d2h_ms_std);
    }
    return RFX_OK;
}

int copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind)
{
    if (bytes == 0) {
        return RFX_OK;
    }
    const cudaError_t err = cudaMemcpy(dst, src, bytes, kind);
    return err == cudaSuccess ? RFX_OK : cuda_fail(err, "cudaMemcpy");
}

}  // namespace

extern "C" {

int rfx_fir_host(int impl, const void* x_iq, int64_t num_samples, const float* taps,
                 int num_taps, int block, void* y_iq, rfx_bench* bench)
{
    return rfx_fir_host_format(impl, RFX_FORMAT_CF32, x_iq, num_samples, taps, num_taps, block,
                               y_iq, bench);
}

int rfx_fir_host_format(int impl, int format, const void* x_iq, int64_t num_samples,
                        const float* taps, int num_taps, int block, void* y_iq, rfx_bench* bench)
{
    if (block < 32 || block > 1024 || block % 32 != 0) {
        return fail(RFX_ERR_INVALID, "--block needs a multiple of 32 up to 1024, got %d", block);
    }
    if (check_format(format) != RFX_OK) {
        return RFX_ERR_INVALID;
    }
    if (num_samples > 0 && (x_iq == nullptr || y_iq == nullptr || taps == nullptr)) {
        return fail(RFX_ERR_INVALID, "fir: null host pointer");
    }
    DeviceMem dx, dy, dh;
    const size_t xbytes = static_cast<size_t>(num_samples) * format_sample_bytes(format);
    const size_t ybytes = static_cast<size_t>(num_samples) * 8;
    cudaError_t err;
    if (num_samples > 0) {
        if ((err = cudaMalloc(&dx.p, xbytes)) != cudaSuccess ||
            (err = cudaMalloc(&dy.p, ybytes)) != cudaSuccess) {
            return cuda_fail(err, "cudaMalloc");
        }
    }
    if (num_taps > 0 && (err = cudaMalloc(&dh.p, sizeof(float) * num_taps)) != cudaSuccess) {
        return cuda_fail(err, "cudaMalloc");
    }
    int rc = check_fir_args(impl, dx.p, static_cast<const float*>(dh.p), dy.p, num_samples,
                            num_taps);
    if (rc != RFX_OK) {
        return rc;
    }
    return timed_passes(
        bench,
        [&] {
            int r = copy(dx.p, x_iq, xbytes, cudaMemcpyHostToDevice);
            return r != RFX_OK ? r
                               : copy(dh.p, taps, sizeof(float) * num_taps,
                                      cudaMemcpyHostToDevice);
        },
        [&] {
            return rfx_fir_launch_format(impl, format, dx.p, static_cast<const float*>(dh.p),
                                         dy.p, num_samples, num_taps, nullptr);
        },
        [&] { return copy(y_iq, dy.p, ybytes, cudaMemcpyDeviceToHost); });
}

int rfx_channelize_host(int impl, const void* x_iq, int64_t num_samples, const float* taps,
                        int num_taps, int channels, void* z_iq, rfx_bench* bench)
{
    return rfx_channelize_host_format(impl, RFX_FORMAT_CF32, RFX_CHAN_OUT_COMPLEX, x_iq,
                                      num_samples, taps, num_taps, channels, z_iq, bench);
}

int rfx_channelize_host_format(int impl, int format, int output, const void* x,
                               int64_t num_samples, const float* taps, int num_taps,
                               int channels, void* out, rfx_bench* bench)
{
    if (check_format(format) != RFX_OK) {
        return RFX_ERR_INVALID;
    }
    if (output != RFX_CHAN_OUT_COMPLEX && output != RFX_CHAN_OUT_MAGNITUDE) {
        return fail(RFX_ERR_INVALID, "channelize: unknown output %d", output);
    }
    if (channels < 1) {
        return fail(RFX_ERR_INVALID, "channelize: need at least one channel");
    }
    if (num_taps < 1) {
        return fail(RFX_ERR_INVALID, "channelize: need at least one tap");
    }
    const int64_t frames = rfx_channelize_frames(num_samples, channels);
    if (frames == 0) {
        return RFX_OK;
    }
    if (x == nullptr || out == nullptr || taps == nullptr) {
        return fail(RFX_ERR_INVALID, "channelize: null host pointer");
    }
    rfx_chan_plan* plan = nullptr;
    int rc = rfx_chan_plan_create(impl, channels, num_samples, &plan);
    if (rc != RFX_OK) {
        return rc;
    }
    struct PlanGuard {
        rfx_chan_plan* p;
        ~PlanGuard() { rfx_chan_plan_destroy(p); }
    } guard{plan};
    DeviceMem dx, dz, dh;
    const size_t xbytes = static_cast<size_t>(num_samples) * format_sample_bytes(format);
    const size_t zbytes = static_cast<size_t>(frames) * channels *
                          (output == RFX_CHAN_OUT_MAGNITUDE ? 4u : 8u);
    cudaError_t err;
    if ((err = cudaMalloc(&dx.p, xbytes)) != cudaSuccess ||
        (err = cudaMalloc(&dz.p, zbytes)) != cudaSuccess ||
        (err = cudaMalloc(&dh.p, sizeof(float) * num_taps)) != cudaSuccess) {
        return cuda_fail(err, "cudaMalloc");
    }
    return timed_passes(
        bench,
        [&] {
            int r = copy(dx.p, x, xbytes, cudaMemcpyHostToDevice);
            return r != RFX_OK ? r
                               : copy(dh.p, taps, sizeof(float) * num_taps,
                                      cudaMemcpyHostToDevice);
        },
        [&] {
            return rfx_channelize_launch_format(plan, format, output, dx.p,
                                                static_cast<const float*>(dh.p), dz.p,
                                                num_samples, num_taps, nullptr);
        },
        [&] { return copy(out, dz.p, zbytes, cudaMemcpyDeviceToHost); });
}

int rfx_magnitude_host(const void* x_iq, int64_t num_samples, float* mag, rfx_bench* bench)
{
    if (num_samples < 0 || num_samples > kMaxSamples) {
        return fail(RFX_ERR_INVALID, "magnitude: %lld samples, expected 0 to %lld",
                    static_cast<long long>(num_samples), static_cast<long long>(kMaxSamples));
    }
    if (num_samples == 0) {
        return RFX_OK;
    }
    if (x_iq == nullptr || mag == nullptr) {
        return fail(RFX_ERR_INVALID, "magnitude: null host pointer");
    }
    DeviceMem dx, dm;
    const size_t xbytes = static_cast<size_t>(num_samples) * 8;
    const size_t mbytes = static_cast<size_t>(num_samples) * 4;
    cudaError_t err;
    if ((err = cudaMalloc(&dx.p, xbytes)) != cudaSuccess ||
        (err = cudaMalloc(&dm.p, mbytes)) != cudaSuccess) {
        return cuda_fail(err, "cudaMalloc");
    }
    return timed_passes(
        bench, [&] { return copy(dx.p, x_iq, xbytes, cudaMemcpyHostToDevice); },
        [&] { return rfx_magnitude_launch(dx.p, static_cast<float*>(dm.p), num_samples, nullptr); },
        [&] { return copy(mag, dm.p, mbytes, cudaMemcpyDeviceToHost); });
}

int rfx_channelize_magnitude_host(int impl, const void* x_iq, int64_t num_samples,
                                  const float* taps, int num_taps, int channels, float* mag,
                                  rfx_bench* bench)
{
    return rfx_channelize_host_format(impl, RFX_FORMAT_CF32, RFX_CHAN_OUT_MAGNITUDE, x_iq,
                                      num_samples, taps, num_taps, channels, mag, bench);
}

}  // extern "C"
