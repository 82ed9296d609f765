// rfx_channelize_tc_static: the 64-channel tensor-core channelizer without a plan and without
// any allocation.
//
// The tensor-core channelizer multiplies by a twiddle operand (the 64-point inverse DFT as a
// 128 x 128 real matrix, FP16 hi and lo images in the MMA's shared-memory layout: 66,048
// bytes). rfx_chan_plan_create allocates it with cudaMalloc and builds it once per plan. This
// entry point keeps it instead in a fixed array of the library's device memory (below), built
// by the first call on each device, so that a caller needs no plan and the library allocates
// nothing. It is for callers that may not allocate device memory after start-up: processing
// loops with a memory budget fixed at initialization, code running under another framework's
// device allocator, or code that must not take the implicit synchronization of cudaMalloc and
// cudaFree.
#include "rfx.h"

#include "api_error.hpp"
#include "chan_tc.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

namespace rfx {
namespace {

constexpr int kStaticChannels = 64;
// 2 images (hi, lo) x 16 planes of 8 K-elements x (128 rows x 16 B + 16 B): the operand of the
// 64-channel form, the only channel count the tensor-core channelizer takes.
constexpr size_t kStaticTwiddleBytes = 66048;
constexpr int kMaxDevices = 64;

// Shared by every call on a device. Written only by that device's first call (zeroed, then
// the twiddle kernel), read-only afterwards.
static __device__ __align__(256) unsigned char g_static_twiddles[kStaticTwiddleBytes];

std::mutex g_setup_mutex;
// Per device: the array's device address and the id of the CUDA context it was built in. A
// cudaDeviceReset destroys that context and reloads the module with the array zeroed; the next
// call sees a new context id and builds the operand again.
void* g_twiddles_of[kMaxDevices];
unsigned long long g_context_of[kMaxDevices];

using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);

// The unique id of the calling thread's current CUDA context (0 if there is none), through the
// driver entry points the runtime hands out (no link against libcuda).
unsigned long long current_context_id()
{
    static CtxGetCurrent get_current = nullptr;
    static CtxGetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa{}, qb{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault,
                                             &qa) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) ==
                cudaSuccess &&
            qb == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<CtxGetCurrent>(a);
            get_id = reinterpret_cast<CtxGetId>(b);
        }
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current == nullptr || get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr ||
        get_id(ctx, &id) != CUDA_SUCCESS) {
        return 0;
    }
    return id;
}

int cuda_error(cudaError_t err, const char* where)
{
    char msg[256];
    std::snprintf(msg, sizeof(msg), "CUDA error: %s (code %d) in %s", cudaGetErrorString(err),
                  static_cast<int>(err), where);
    return set_last_error(RFX_ERR_CUDA, msg);
}

// Builds the twiddle image in the static array of the current device on the first call in this
// CUDA context (the image's unused padding must be zero, so the array is cleared first), then
// waits for it on `stream`, so that calls on any stream of the device see the finished image.
int static_twiddles(int device, cudaStream_t stream, void** out)
{
    // The array's address in this context; this also makes the device's primary context
    // current, so that the context id below is the one the kernel will run in.
    void* p = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&p, g_static_twiddles);
    if (err != cudaSuccess) {
        return cuda_error(err, "channelize_tc_static setup (cudaGetSymbolAddress)");
    }
    const unsigned long long context = current_context_id();
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_twiddles_of[device] == p && context != 0 && g_context_of[device] == context) {
        *out = p;
        return RFX_OK;
    }
    if (chan_tc_twiddle_bytes() > kStaticTwiddleBytes) {
        return set_last_error(RFX_ERR_CAPACITY,
                              "channelize_tc_static: the twiddle operand outgrew the static array");
    }
    // The build is stream work followed by a wait: inside a stream capture it would be
    // recorded into the caller's graph and the wait would break the capture.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    err = cudaStreamIsCapturing(stream, &capture);
    if (err != cudaSuccess) {
        return cuda_error(err, "channelize_tc_static setup (cudaStreamIsCapturing)");
    }
    if (capture != cudaStreamCaptureStatusNone) {
        return set_last_error(RFX_ERR_INVALID,
                              "channelize_tc_static: the first call on a device (and the first "
                              "after cudaDeviceReset) builds the twiddle operand and must be "
                              "made outside stream capture");
    }
    err = chan_tc_build_twiddles(p, stream);
    if (err == cudaSuccess) {
        err = cudaStreamSynchronize(stream);
    }
    if (err != cudaSuccess) {
        return cuda_error(err, "channelize_tc_static setup");
    }
    g_twiddles_of[device] = p;
    g_context_of[device] = context;
    *out = p;
    return RFX_OK;
}

}  // namespace
}  // namespace rfx

extern "C" int rfx_channelize_tc_static(const void* x, const float* taps, void* out,
                                        int64_t num_samples, int num_taps, int channels,
                                        cudaStream_t stream)
{
    using namespace rfx;
    char msg[256];
    if (channels != kStaticChannels) {
        std::snprintf(msg, sizeof(msg),
                      "channelize_tc_static: %d channels; the static twiddle array (%zu bytes) "
                      "holds the operand of 64 channels only",
                      channels, kStaticTwiddleBytes);
        return set_last_error(channels < 1 ? RFX_ERR_INVALID : RFX_ERR_CAPACITY, msg);
    }
    if (num_samples < 0 || num_samples > INT32_MAX) {
        std::snprintf(msg, sizeof(msg), "channelize_tc_static: %lld samples, expected 0 to %d",
                      static_cast<long long>(num_samples), INT32_MAX);
        return set_last_error(RFX_ERR_INVALID, msg);
    }
    if (num_taps < 1) {
        return set_last_error(RFX_ERR_INVALID, "channelize_tc_static: need at least one tap");
    }
    if (num_samples == 0) {
        return RFX_OK;
    }
    if (num_samples < kStaticChannels) {
        return set_last_error(RFX_ERR_INVALID,
                              "channelize_tc_static: needs at least one full frame (64 samples)");
    }
    if (x == nullptr || taps == nullptr || out == nullptr) {
        return set_last_error(RFX_ERR_INVALID, "channelize_tc_static: null pointer");
    }
    if ((reinterpret_cast<uintptr_t>(x) & 15u) != 0 ||
        (reinterpret_cast<uintptr_t>(out) & 15u) != 0) {
        return set_last_error(RFX_ERR_ALIGNMENT,
                              "channelize_tc_static: sample buffers must be 16-byte aligned");
    }
    if (!chan_tc_supported(kStaticChannels, num_taps)) {
        std::snprintf(msg, sizeof(msg),
                      "channelize_tc_static: %d taps exceed the tensor-core form's shared memory",
                      num_taps);
        return set_last_error(RFX_ERR_CAPACITY, msg);
    }
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess || device < 0 || device >= kMaxDevices) {
        return set_last_error(RFX_ERR_CUDA, "channelize_tc_static: no usable current device");
    }
    void* twiddles = nullptr;
    const int status = static_twiddles(device, stream, &twiddles);
    if (status != RFX_OK) {
        return status;
    }
    err = chan_tc_launch(x, taps, twiddles, out, num_samples, num_taps, stream);
    return err == cudaSuccess ? RFX_OK : cuda_error(err, "chan_tc_launch");
}
