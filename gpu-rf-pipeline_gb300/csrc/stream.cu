// rfx_fir_stream: the FIR of a host capture in chunks, the way live radio data arrives, with the
// transfers of one chunk overlapping the kernel of another (src/stream.hpp:1-26,
// src/stream.cu:135-222).
//
// `depth` slots form a ring; each has pinned host buffers (copy and zero-copy modes), device
// buffers, its own CUDA stream and an event. Chunk i goes to slot i % depth: the host waits for
// that slot's previous chunk, fills the slot, and enqueues upload, kernel and download on the
// slot's stream, so the two copy engines and the SMs work on different chunks at once.
//
// Every chunk is computed together with history, so that the streamed output carries the same
// bits as one run over the whole capture with the same implementation:
//  * plain kernel: each output is one fused multiply-add chain over its K inputs, so the chunk
//    plus K - 1 samples of history suffices (as the project);
//  * tensor-core form: a tile's results depend on its tile-wide scale, i.e. on the samples from
//    its window start to its end. The chunk's outputs are computed as whole tiles at the
//    capture's absolute tile positions (the computed stretch is widened to tile boundaries and
//    one tile of history is added), so every kept output comes from the same tile as in the
//    whole run;
//  * the implementation (auto resolved once for the whole capture) and the tensor-core tile
//    shape and ring depth are fixed before the first chunk.
//
// Input formats: cf32, or integer I/Q as stored (ci16, ci8: rfx_sample_format) — then only the
// stored bytes cross the host link and the kernels convert them in their load stage, with the
// bits of streaming the converted samples (integer input runs the single-CTA tensor-core form,
// whose tile the chunking follows).
//
// Memory modes (src/stream.hpp:34-38): copy (host copies into and out of the pinned ring);
// registered (x and y page-locked in place; memory that is already page-locked is used as is);
// zero-copy (the chunk is written into mapped pinned memory, a gather kernel reads it across the
// bus into the slot's device buffer, and a scatter kernel writes the outputs back into mapped
// memory: no cudaMemcpy, the same bus traffic as a kernel reading host memory directly; the
// filter kernels themselves stage through TMA and need device-resident operands).
#include "rfx.h"

#include "api_error.hpp"
#include "fir_plain.cuh"
#include "fir_tc.cuh"
#include "tuning.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <vector>

namespace rfx {
namespace {

template <typename T>
__global__ void copy_elements(const T* __restrict__ src, T* __restrict__ dst, long long n)
{
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    for (long long i = static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += stride) {
        dst[i] = src[i];
    }
}

// Copies n samples of `sample_bytes` bytes (8, 4 or 2) with one element per sample.
cudaError_t launch_copy(const void* src, void* dst, long long n, int sample_bytes,
                        cudaStream_t stream)
{
    if (n <= 0) {
        return cudaSuccess;
    }
    const unsigned blocks = static_cast<unsigned>(std::min<long long>((n + 255) / 256, 4096));
    if (sample_bytes == 8) {
        copy_elements<<<blocks, 256, 0, stream>>>(static_cast<const float2*>(src),
                                                  static_cast<float2*>(dst), n);
    } else if (sample_bytes == 4) {
        copy_elements<<<blocks, 256, 0, stream>>>(static_cast<const unsigned int*>(src),
                                                  static_cast<unsigned int*>(dst), n);
    } else {
        copy_elements<<<blocks, 256, 0, stream>>>(static_cast<const unsigned short*>(src),
                                                  static_cast<unsigned short*>(dst), n);
    }
    return cudaGetLastError();
}

int cuda_error(cudaError_t err, const char* what)
{
    char msg[256];
    std::snprintf(msg, sizeof(msg), "CUDA error: %s (code %d) in %s", cudaGetErrorString(err),
                  static_cast<int>(err), what);
    return set_last_error(RFX_ERR_CUDA, msg);
}

struct Slot {
    void* host_in = nullptr;    // pinned (mapped in zero-copy mode)
    void* host_out = nullptr;
    void* dev_in = nullptr;
    void* dev_out = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    long long start = 0;   // the chunk's outputs: y[start, start + count), at `offset` in dev_out
    long long count = 0;
    long long offset = 0;
    bool busy = false;
};

// Everything the run allocates, released on every exit path.
struct Resources {
    std::vector<Slot> slots;
    float* taps = nullptr;
    const void* registered[2] = {nullptr, nullptr};

    ~Resources()
    {
        for (Slot& s : slots) {
            if (s.stream != nullptr) {
                cudaStreamSynchronize(s.stream);
                cudaStreamDestroy(s.stream);
            }
            if (s.done != nullptr) {
                cudaEventDestroy(s.done);
            }
            cudaFreeHost(s.host_in);
            cudaFreeHost(s.host_out);
            cudaFree(s.dev_in);
            cudaFree(s.dev_out);
        }
        cudaFree(taps);
        for (const void* p : registered) {
            if (p != nullptr) {
                cudaHostUnregister(const_cast<void*>(p));
            }
        }
    }
};

// Page-locks [p, p + bytes) unless it already is; records what it registered.
cudaError_t lock_in_place(const void* p, size_t bytes, const void** registered)
{
    cudaPointerAttributes attr{};
    if (cudaPointerGetAttributes(&attr, p) == cudaSuccess && attr.type == cudaMemoryTypeHost) {
        return cudaSuccess;  // already pinned
    }
    cudaGetLastError();
    const cudaError_t err = cudaHostRegister(const_cast<void*>(p), bytes, cudaHostRegisterDefault);
    if (err == cudaErrorHostMemoryAlreadyRegistered) {
        cudaGetLastError();
        return cudaSuccess;
    }
    if (err == cudaSuccess) {
        *registered = p;
    }
    return err;
}

}  // namespace
}  // namespace rfx

extern "C" int rfx_fir_stream(const void* x_iq, int64_t num_samples, const float* taps,
                              int num_taps, const rfx_stream_config* config, void* y_iq,
                              double* total_ms, int* chunks_out)
{
    return rfx_fir_stream_format(RFX_FORMAT_CF32, x_iq, num_samples, taps, num_taps, config,
                                 y_iq, total_ms, chunks_out);
}

extern "C" int rfx_fir_stream_format(int format, const void* x_in, int64_t num_samples,
                                     const float* taps, int num_taps,
                                     const rfx_stream_config* config, void* y_iq,
                                     double* total_ms, int* chunks_out)
{
    using namespace rfx;
    char msg[256];
    if (format < RFX_FORMAT_CF32 || format > RFX_FORMAT_CI8) {
        std::snprintf(msg, sizeof(msg), "stream: unknown sample format %d", format);
        return set_last_error(RFX_ERR_INVALID, msg);
    }
    // Bytes per input sample as stored: cf32 8, ci16 4, ci8 2 (outputs are cf32).
    const int ib = format == RFX_FORMAT_CF32 ? 8 : format == RFX_FORMAT_CI16 ? 4 : 2;
    if (config == nullptr) {
        return set_last_error(RFX_ERR_INVALID, "stream: null config");
    }
    if (config->chunk < 1 || config->depth < 1) {
        return set_last_error(RFX_ERR_INVALID, "stream: chunk and depth must be at least 1");
    }
    if (config->memory < RFX_STREAM_COPY || config->memory > RFX_STREAM_ZERO_COPY) {
        std::snprintf(msg, sizeof(msg), "stream: unknown memory mode %d", config->memory);
        return set_last_error(RFX_ERR_INVALID, msg);
    }
    if (config->impl < RFX_FIR_PLAIN || config->impl > RFX_FIR_AUTO) {
        std::snprintf(msg, sizeof(msg), "stream: unknown implementation %d", config->impl);
        return set_last_error(RFX_ERR_INVALID, msg);
    }
    if (num_samples < 0 || num_samples > INT32_MAX ||
        config->chunk + num_taps > static_cast<int64_t>(INT32_MAX)) {
        return set_last_error(RFX_ERR_INVALID, "stream: sample counts beyond 2^31 - 1");
    }
    if (num_taps < 1 || num_taps > kMaxTaps) {
        std::snprintf(msg, sizeof(msg), "stream: %d taps, expected 1 to %d", num_taps, kMaxTaps);
        return set_last_error(num_taps < 1 ? RFX_ERR_INVALID : RFX_ERR_CAPACITY, msg);
    }
    if (total_ms != nullptr) {
        *total_ms = 0.0;
    }
    if (chunks_out != nullptr) {
        *chunks_out = 0;
    }
    if (num_samples == 0) {
        return RFX_OK;
    }
    if (x_in == nullptr || y_iq == nullptr || taps == nullptr) {
        return set_last_error(RFX_ERR_INVALID, "stream: null host pointer");
    }

    // The implementation and tile geometry of the whole run, fixed for every chunk.
    const long long n = num_samples;
    int impl = config->impl;
    if (impl == RFX_FIR_AUTO) {
        impl = tuned_fir_impl(num_taps, n);
    }
    if (impl == RFX_FIR_TC && !fir_tc_supported(num_taps)) {
        impl = RFX_FIR_PLAIN;  // as rfx_fir_launch: one tap, or beyond the tensor-core form
    }
    const TcConfig tc = tuned_fir_tc_config(num_taps, n);
    const long long tile =
        impl == RFX_FIR_TC ? fir_tc_tile_outputs_format(format, num_taps, n, tc) : 1;
    const long long history = tile > 1 ? tile : num_taps - 1;
    const long long chunk = config->chunk;
    const long long slot_len = chunk + 2 * (tile - 1) + history;
    const int memory = config->memory;
    const bool registered = memory == RFX_STREAM_REGISTERED;
    const bool zero_copy = memory == RFX_STREAM_ZERO_COPY;

    // Setup, outside the clock.
    Resources res;
    cudaError_t err;
    res.slots.resize(static_cast<size_t>(config->depth));
    const size_t slot_bytes = static_cast<size_t>(slot_len) * 8;
    const size_t slot_in_bytes = static_cast<size_t>(slot_len) * ib;
    for (Slot& s : res.slots) {
        if (!registered) {
            const unsigned flags = zero_copy ? cudaHostAllocMapped : cudaHostAllocDefault;
            if ((err = cudaHostAlloc(&s.host_in, slot_in_bytes, flags)) != cudaSuccess ||
                (err = cudaHostAlloc(&s.host_out, slot_bytes, flags)) != cudaSuccess) {
                return cuda_error(err, "stream: cudaHostAlloc");
            }
        }
        if ((err = cudaMalloc(&s.dev_in, slot_in_bytes)) != cudaSuccess ||
            (err = cudaMalloc(&s.dev_out, slot_bytes)) != cudaSuccess ||
            (err = cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (err = cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming)) != cudaSuccess) {
            return cuda_error(err, "stream: slot setup");
        }
    }
    const size_t bytes = static_cast<size_t>(n) * 8;
    if (registered) {
        if ((err = lock_in_place(x_in, static_cast<size_t>(n) * ib, &res.registered[0])) !=
                cudaSuccess ||
            (err = lock_in_place(y_iq, bytes, &res.registered[1])) != cudaSuccess) {
            return cuda_error(err, "stream: cudaHostRegister");
        }
    }
    if ((err = cudaMalloc(&res.taps, sizeof(float) * num_taps)) != cudaSuccess ||
        (err = cudaMemcpy(res.taps, taps, sizeof(float) * num_taps, cudaMemcpyHostToDevice)) !=
            cudaSuccess ||
        (err = cudaDeviceSynchronize()) != cudaSuccess) {
        return cuda_error(err, "stream: tap upload");
    }

    const auto* x = static_cast<const unsigned char*>(x_in);   // samples of ib bytes
    auto* y = static_cast<float2*>(y_iq);
    // Waits for the chunk in `s`, then moves its outputs into y (copy and zero-copy modes).
    auto retire = [&](Slot& s) -> cudaError_t {
        if (!s.busy) {
            return cudaSuccess;
        }
        const cudaError_t e = cudaEventSynchronize(s.done);
        if (e != cudaSuccess) {
            return e;
        }
        if (!registered) {
            std::memcpy(y + s.start, static_cast<float2*>(s.host_out) + s.offset,
                        static_cast<size_t>(s.count) * 8);
        }
        s.busy = false;
        return cudaSuccess;
    };

    const auto begin = std::chrono::steady_clock::now();
    int chunks = 0;
    for (long long start = 0; start < n; start += chunk, ++chunks) {
        Slot& s = res.slots[static_cast<size_t>(chunks % config->depth)];
        if ((err = retire(s)) != cudaSuccess) {
            return cuda_error(err, "stream: chunk completion");
        }
        const long long end = std::min(n, start + chunk);
        // Outputs computed: whole tiles around [start, end); inputs: those plus the history.
        const long long c0 = start / tile * tile;
        const long long c1 = std::min(n, (end + tile - 1) / tile * tile);
        const long long in_start = c0 > history ? c0 - history : 0;
        const long long in_len = c1 - in_start;
        s.start = start;
        s.count = end - start;
        s.offset = start - in_start;
        const cudaStream_t st = s.stream;
        const unsigned char* src_in = x + static_cast<size_t>(in_start) * ib;
        const size_t in_bytes = static_cast<size_t>(in_len) * ib;
        if (registered) {
            err = cudaMemcpyAsync(s.dev_in, src_in, in_bytes, cudaMemcpyHostToDevice, st);
        } else {
            // Where a receiver would write the samples.
            std::memcpy(s.host_in, src_in, in_bytes);
            if (zero_copy) {
                void* mapped = nullptr;
                err = cudaHostGetDevicePointer(&mapped, s.host_in, 0);
                if (err == cudaSuccess) {
                    err = launch_copy(mapped, s.dev_in, in_len, ib, st);
                }
            } else {
                err = cudaMemcpyAsync(s.dev_in, s.host_in, in_bytes, cudaMemcpyHostToDevice, st);
            }
        }
        if (err != cudaSuccess) {
            return cuda_error(err, "stream: upload");
        }
        err = impl == RFX_FIR_TC
                  ? fir_tc_launch_format(format, s.dev_in, res.taps, s.dev_out, in_len, num_taps,
                                         tc, st)
                  : fir_plain_launch_format(format, s.dev_in, res.taps, s.dev_out, in_len,
                                            num_taps, st);
        if (err != cudaSuccess) {
            return cuda_error(err, "stream: FIR launch");
        }
        // Only the chunk's own outputs come back.
        const float2* src = static_cast<const float2*>(s.dev_out) + s.offset;
        const size_t out_bytes = static_cast<size_t>(s.count) * 8;
        if (registered) {
            err = cudaMemcpyAsync(y + start, src, out_bytes, cudaMemcpyDeviceToHost, st);
        } else if (zero_copy) {
            void* mapped = nullptr;
            err = cudaHostGetDevicePointer(&mapped, s.host_out, 0);
            if (err == cudaSuccess) {
                err = launch_copy(src, static_cast<float2*>(mapped) + s.offset, s.count, 8, st);
            }
        } else {
            err = cudaMemcpyAsync(static_cast<float2*>(s.host_out) + s.offset, src, out_bytes,
                                  cudaMemcpyDeviceToHost, st);
        }
        if (err != cudaSuccess || (err = cudaEventRecord(s.done, st)) != cudaSuccess) {
            return cuda_error(err, "stream: download");
        }
        s.busy = true;
    }
    // Drain in chunk order.
    for (int i = 0; i < config->depth; ++i) {
        if ((err = retire(res.slots[static_cast<size_t>((chunks + i) % config->depth)])) !=
            cudaSuccess) {
            return cuda_error(err, "stream: chunk completion");
        }
    }
    const auto finish = std::chrono::steady_clock::now();
    if (total_ms != nullptr) {
        *total_ms = std::chrono::duration<double, std::milli>(finish - begin).count();
    }
    if (chunks_out != nullptr) {
        *chunks_out = chunks;
    }
    return RFX_OK;
}
