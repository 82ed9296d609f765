/*
 * rfx.h — C ABI of the GB300-native complex-baseband filtering library (librfx.so).
 *
 * The library replaces the hot path of the gpu-rf-pipeline project: the complex-float32 FIR
 * filter (src/fir.cu) and the critically sampled polyphase channelizer (src/channelize.cu),
 * behind the project's device-pointer entry points (src/device_ops.hpp) and its host-vector
 * operations (src/ops.hpp). Every function here names the project interface it replaces.
 *
 * Conventions (all functions):
 *   - Plain C types only. A cf32 sample is two little-endian float32 values, I then Q
 *     (src/types.hpp:7-12); `x`, `y`, `out` point to arrays of them.
 *   - Device pointers must be 16-byte aligned (cudaMalloc and PyTorch allocations are).
 *   - Lengths are 64-bit. The FIR and the channelizer accept up to 2^31 - 1 samples per call.
 *   - Every function returns an rfx_status; RFX_OK is 0. On failure, rfx_last_error() returns a
 *     message for the calling thread. The C++ layer above maps non-zero statuses to
 *     std::runtime_error, as the project's CUDA_CHECK does (src/check.hpp:42-66).
 *   - The launch functions only enqueue work on the given stream (0 = the legacy default
 *     stream): no allocation, no host transfer, no synchronization (src/device_ops.hpp:3-7).
 *   - Device-side waits inside the kernels are bounded. A kernel that gives up records a fault
 *     code that rfx_device_fault() reports; the CUDA context stays usable.
 */
#ifndef RFX_H
#define RFX_H

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rfx_status {
    RFX_OK = 0,
    RFX_ERR_INVALID = 1,     /* bad argument (null pointer, negative length, no taps ...) */
    RFX_ERR_CAPACITY = 2,    /* valid but beyond what the chosen implementation supports */
    RFX_ERR_ALIGNMENT = 3,   /* a device pointer is not 16-byte aligned */
    RFX_ERR_CUDA = 4,        /* a CUDA runtime or cuFFT call failed */
    RFX_ERR_DEVICE_FAULT = 5 /* a kernel gave up on a bounded wait (see rfx_device_fault) */
} rfx_status;

/* FIR implementations (values of `impl`). */
typedef enum rfx_fir_impl {
    /* FP32 CUDA-core kernel: sample tile staged in shared memory by the bulk-copy (TMA) engine,
     * nine outputs per thread from a register window, packed f32x2 fused multiply-adds.
     * Same arithmetic as the project's naive/tiled/register kernels (one fused multiply-add
     * per tap, taps in ascending order), so results are bit-identical to theirs. */
    RFX_FIR_PLAIN = 0,
    /* Tensor-core kernel (tcgen05): the FIR as a block-Toeplitz GEMM in split FP16
     * (hi + lo operands, three products, FP32 accumulation in tensor memory) with one
     * power-of-two scale per tile. Tolerance-tested, not bit-exact. Calls it cannot take run
     * RFX_FIR_PLAIN instead: one tap, more than 3457 taps (the shared-memory budget), fewer
     * than 128 samples; rfx_fir_impl_used() says in advance which kernel a call runs. */
    RFX_FIR_TC = 1,
    /* Chooses per call from the tuned table (rfx_autotune) or a built-in rule. */
    RFX_FIR_AUTO = 2
} rfx_fir_impl;

/* Channelizer implementations. */
typedef enum rfx_chan_impl {
    /* FP32 branch-sum kernel (bit-identical to the project's channelize_branch_kernel) followed
     * by cuFFT's batched in-place inverse transform, as the project computes it. */
    RFX_CHAN_PLAIN = 0,
    /* The M-point DFT as a split-FP16 complex GEMM on tcgen05. M = 64: one fused kernel (FP32
     * branch sums into shared memory, then the GEMM). M = 1024: the plain form's FP32 branch
     * sums, then the DFT factored 32 x 32 into two GEMMs with an FP32 twiddle between them. */
    RFX_CHAN_TC = 1,
    /* Chosen when the plan is made, from the tuned table (rfx_autotune_channelize) or the
     * built-in rule (the tensor-core form at 64 channels, the plain form otherwise). */
    RFX_CHAN_AUTO = 2
} rfx_chan_impl;

/* ---- errors and identification -------------------------------------------------------- */

/* Message of the calling thread's last failed call ("" if none). */
const char* rfx_last_error(void);

/* Synchronizes the current device, returns the fault code any kernel of this library recorded
 * since the last call (0 = none) and clears it. */
int rfx_device_fault(unsigned int* code);

/* Library version, e.g. "rfx 0.1.0 sm_103a". */
const char* rfx_version(void);

/* Implementation names for `rfgpu info` and --impl: writes at most `size` bytes of the name of
 * implementation `index` into `name`; returns RFX_ERR_INVALID past the last one.
 * Replaces fir_impls() (src/ops.hpp:36, table at src/fir.cu:725-734). */
int rfx_fir_impl_name(int index, char* name, size_t size);
int rfx_chan_impl_name(int index, char* name, size_t size);

/* Parses an --impl name into an rfx_fir_impl. Accepts "plain", "tc_split", "auto" and, as
 * aliases of "plain" (same results bit for bit), the project's "naive", "tiled",
 * "tiled_const" and "register". Replaces parse_fir_impl (src/device_ops.hpp:75). */
int rfx_parse_fir_impl(const char* name, int* impl);
int rfx_parse_chan_impl(const char* name, int* impl);

/* ---- FIR, device pointers ------------------------------------------------------------- */

/* y[n] = sum_k taps[k] x[n - k] for 0 <= n < num_samples, x[m < 0] = 0; `taps` in GPU memory
 * (num_taps <= 8192). Enqueued on `stream`.
 * Replaces fir_launch (src/device_ops.hpp:88-89). */
int rfx_fir_launch(int impl, const void* x, const float* taps, void* y, int64_t num_samples,
                   int num_taps, cudaStream_t stream);

/* Which kernel rfx_fir_launch (batch == 0) or rfx_fir_batch_launch (batch != 0, for one
 * capture) runs for these arguments: writes RFX_FIR_PLAIN or RFX_FIR_TC to *used. Resolves
 * RFX_FIR_AUTO through the tuned table, and reports where RFX_FIR_TC hands a call to the plain
 * kernel (see RFX_FIR_TC; the batch kernel's budget is smaller). Host-only, no GPU work.
 * No counterpart in the project, whose --impl always names the kernel that runs. */
int rfx_fir_impl_used(int impl, int num_taps, int64_t num_samples, int batch, int* used);

/* rfx_fir_launch on the legacy default stream. Replaces fir_device (src/device_ops.hpp:81-82). */
int rfx_fir_device(int impl, const void* x, const float* taps, void* y, int64_t num_samples,
                   int num_taps);

/* Sample formats of an input buffer: the SigMF datatypes the project reads
 * (src/io.cpp:126-148), interleaved I/Q, little-endian. */
typedef enum rfx_sample_format {
    RFX_FORMAT_CF32 = 0,  /* cf32_le: float32 components */
    RFX_FORMAT_CI16 = 1,  /* ci16_le: int16 components, each read as v / 32768 */
    RFX_FORMAT_CI8 = 2    /* ci8 / ci8_le: int8 components, each read as v / 128 */
} rfx_sample_format;

/* rfx_fir_launch over x stored in `format` (num_samples samples of 8, 4 or 2 bytes), converted
 * in the kernels' load stage instead of on the host: the same results as converting every
 * sample as the project's SigMF reader does (src/io.cpp:110-124) and calling rfx_fir_launch, for
 * a quarter (ci8) or half (ci16) of the input bytes. RFX_FIR_TC runs its single-CTA form on
 * integer input. y is cf32; x and y 16-byte aligned.
 * No counterpart in the project, which converts on the host before the upload (src/io.cpp:175-181
 * then fir_host). */
int rfx_fir_launch_format(int impl, int format, const void* x, const float* taps, void* y,
                          int64_t num_samples, int num_taps, cudaStream_t stream);

/* Checks that `num_taps` fits the tap capacity. The kernels here read the taps from the pointer
 * passed to each launch, so there is no constant bank to fill: callers that load it first and
 * then launch (src/stream.cu:158-160, :195-202) get the same results.
 * Replaces fir_load_const_taps (src/device_ops.hpp:87). */
int rfx_fir_load_const_taps(const float* taps, int num_taps, cudaStream_t stream);

/* `count` channels sharing one set of taps, in one launch; `x`, `y` and `num_samples` are HOST
 * arrays of `count` entries (device pointers / lengths). No limit of 8 channels.
 * Replaces fir_batched_device (src/device_ops.hpp:99-100). */
int rfx_fir_batched_device(int impl, const void* const* x, void* const* y,
                           const int64_t* num_samples, int count, const float* taps,
                           int num_taps, cudaStream_t stream);

/* One capture of a per-capture-taps batch. */
typedef struct rfx_fir_capture {
    const void* x;          /* device, cf32 */
    void* y;                /* device, cf32 */
    const float* taps;      /* device, float32 */
    int64_t num_samples;
    int32_t num_taps;
    int32_t reserved;       /* must be 0 */
} rfx_fir_capture;

/* Up to 4096 captures, each with its own taps, in ONE persistent launch (a work list of
 * (capture, tile) items). `captures` is a HOST array. No counterpart in the project, which
 * runs such a batch as one fir_launch per capture (src/stream.cu:195-202 pattern). */
int rfx_fir_batch_launch(int impl, const rfx_fir_capture* captures, int count,
                         cudaStream_t stream);

/* A batch plan: the work list of one batch of captures (each with its own taps) built once in
 * device memory — capture tables, TMA tensor maps, each block's share of the work — so that
 * every run of the batch is ONE persistent kernel launch, replayable from a CUDA graph. The
 * launch takes every capture of the batch: those the implementation puts on the tensor cores
 * (RFX_FIR_TC: all it can take; RFX_FIR_AUTO: as the tuned table or the built-in rule places
 * each capture: every filter of 2 taps or more by the built-in rule) run the block-Toeplitz
 * pipelines (the resident-window phases for 2 to 385 taps, the long-filter tiles beyond), the
 * others (one tap, shorter than 128 samples, beyond the kernel's tap budget, or everything
 * under RFX_FIR_PLAIN) run the plain kernel's tile function with groups of the same blocks'
 * threads, with its bits.
 * The blocks are given contiguous shares of tensor-core tiles and plain tiles of about equal
 * cost, so tensor-bound and memory-bound work run side by side on different SMs.
 * Create allocates and copies (setup; call outside timed regions and stream capture); the
 * capture pointers are bound at creation (the buffers' contents may change between runs).
 * No counterpart in the project, which runs such a batch as one fir_launch per capture, and
 * whose fir_batched_device (src/fused.cu:92-109) takes at most 8 channels sharing one tap set. */
typedef struct rfx_fir_batch_plan rfx_fir_batch_plan;
int rfx_fir_batch_plan_create(int impl, const rfx_fir_capture* captures, int count,
                              rfx_fir_batch_plan** plan);
/* Enqueues the plan's one launch on `stream`; allocates nothing. */
int rfx_fir_batch_run(rfx_fir_batch_plan* plan, cudaStream_t stream);
/* How the plan split the captures, and kernel launches per run (1; 0 for an empty batch). */
int rfx_fir_batch_plan_info(const rfx_fir_batch_plan* plan, int* tc_captures,
                            int* plain_captures, int* launches);
int rfx_fir_batch_plan_destroy(rfx_fir_batch_plan* plan);

/* ---- channelizer ---------------------------------------------------------------------- */

/* ceil(num_samples / channels). Replaces channelize_frames (src/device_ops.hpp:145). */
int64_t rfx_channelize_frames(int64_t num_samples, int channels);

typedef struct rfx_chan_plan rfx_chan_plan;

/* Setup for channelizing up to `max_samples` samples into `channels` channels: for
 * RFX_CHAN_PLAIN, the batched inverse cuFFT plan of `channels` points (the project's FftPlan,
 * src/fft_plan.hpp:15-22); for RFX_CHAN_TC (64 or 1024 channels, RFX_ERR_CAPACITY otherwise),
 * the DFT operand built in FP64 and, at 1024 channels, a buffer for the branch sums
 * (max_samples / 1024 frames x 8 KB). RFX_CHAN_AUTO picks by the tuned table, else the
 * tensor-core form at 64 channels.
 * Allocates; call outside timed regions. */
int rfx_chan_plan_create(int impl, int channels, int64_t max_samples, rfx_chan_plan** plan);
int rfx_chan_plan_destroy(rfx_chan_plan* plan);

/* z[t][k] = sum_l taps[l] x[tM - l] e^{+2 pi i k l / M}, t < ceil(N/M), into `out`
 * (frames * channels cf32, frame-major). `taps` in GPU memory. Enqueued on `stream`.
 * Replaces channelize_device (src/device_ops.hpp:150-151). */
int rfx_channelize_launch(rfx_chan_plan* plan, const void* x, const float* taps, void* out,
                          int64_t num_samples, int num_taps, cudaStream_t stream);

/* The branch sums alone: u[t][m] = sum_p taps[pM + m] x[tM - pM - m] into `u` (frames * channels
 * cf32, frame-major), float32, bit-identical to the project's channelize_branch_kernel
 * (src/channelize.cu:25-49). For callers that run their own inverse FFT on `u`, as the
 * project's channelize_device(cufftHandle, ...) does (src/channelize.cu:56-72). */
int rfx_channelize_branches(const void* x, const float* taps, void* u, int64_t num_samples,
                            int channels, int num_taps, cudaStream_t stream);

/* The channelizer followed by the magnitude of every channel output, mag[t][k] = |z[t][k]|
 * (frames x channels float32). Tensor-core plans compute it in the DFT-GEMM epilogue, so the
 * complex channel outputs never reach HBM; plain plans run the magnitude kernel over the
 * channel outputs in a plan-owned buffer (allocated by the first such call). mag 16-byte
 * aligned. Fuses channelize |> magnitude (compiler/examples/channelizer.sf,
 * src/magnitude.cu:17-25); no single-call counterpart in the project. */
int rfx_channelize_magnitude_launch(rfx_chan_plan* plan, const void* x, const float* taps,
                                    float* mag, int64_t num_samples, int num_taps,
                                    cudaStream_t stream);

/* Outputs of the channelizer entry points that take one. */
typedef enum rfx_chan_output {
    RFX_CHAN_OUT_COMPLEX = 0,    /* z: frames x channels cf32 */
    RFX_CHAN_OUT_MAGNITUDE = 1   /* |z|: frames x channels float32 */
} rfx_chan_output;

/* rfx_channelize_launch / rfx_channelize_magnitude_launch (`output`) over x stored in `format`
 * (rfx_sample_format): integer components are converted where the kernels read the samples,
 * with the results of converting them first as the project does (src/io.cpp:110-148). */
int rfx_channelize_launch_format(rfx_chan_plan* plan, int format, int output, const void* x,
                                 const float* taps, void* out, int64_t num_samples, int num_taps,
                                 cudaStream_t stream);

/* ---- magnitude ------------------------------------------------------------------------- */

/* mag[i] = |x[i]| = sqrt(re^2 + im^2) for i < num_samples (x cf32, mag float32, both 16-byte
 * aligned), enqueued on `stream`. Replaces magnitude_device (src/device_ops.hpp:57,
 * src/magnitude.cu:27-37). */
int rfx_magnitude_launch(const void* x, float* mag, int64_t num_samples, cudaStream_t stream);

/* The 64-channel tensor-core channelizer (what rfx_channelize_launch computes with an
 * RFX_CHAN_TC plan, same kernel and results) without a plan and without allocating anything:
 * its twiddle operand (66,048 bytes) lives in a fixed array of the library's device memory,
 * shared by every call on the device. For callers that may not allocate device memory after
 * start-up: a memory budget fixed at initialization, a device allocator owned by another
 * framework, or no room for the implicit synchronization of cudaMalloc and cudaFree.
 * The FIRST call on each device builds that operand on `stream` and waits for it
 * (cudaStreamSynchronize); make it during initialization, before any stream capture (a first
 * call on a capturing stream returns RFX_ERR_INVALID and leaves the capture intact). Later
 * calls only enqueue the kernel. cudaDeviceReset clears the array; the next call notices the
 * new CUDA context and builds the operand again, as a first call. The array is read-only after the first call, so calls may
 * overlap; concurrent first calls on one device are serialized by a lock.
 * channels must be 64 (RFX_ERR_CAPACITY otherwise: the array holds that operand only);
 * num_samples 0 or at least 64 (one frame); taps as for the RFX_CHAN_TC plan.
 * No counterpart in the project: its channelize_device (src/device_ops.hpp:150-151) takes a
 * cuFFT plan, which allocates. */
int rfx_channelize_tc_static(const void* x, const float* taps, void* out, int64_t num_samples,
                             int num_taps, int channels, cudaStream_t stream);

/* ---- streaming ------------------------------------------------------------------------ */

/* Host memory of a stream run (the project's StreamMemory, src/stream.hpp:34-38). */
typedef enum rfx_stream_memory {
    RFX_STREAM_COPY = 0,        /* samples copied into and out of a pinned ring on the host */
    RFX_STREAM_REGISTERED = 1,  /* x and y page-locked in place (already pinned memory as is) */
    RFX_STREAM_ZERO_COPY = 2    /* chunks moved through mapped pinned memory by GPU kernels */
} rfx_stream_memory;

/* The project's StreamConfig (src/stream.hpp:40-45). */
typedef struct rfx_stream_config {
    int impl;          /* rfx_fir_impl (auto is resolved once, for the whole capture) */
    int memory;        /* rfx_stream_memory */
    int64_t chunk;     /* samples per chunk, >= 1 */
    int depth;         /* slots in the ring (and CUDA streams), >= 1 */
} rfx_stream_config;

/* The FIR of a HOST capture in chunks through a ring of `depth` slots, each chunk's upload,
 * kernel and download on the slot's own stream. `y_iq` receives exactly the bits one
 * rfx_fir_launch of the same implementation over the whole capture would give (each chunk is
 * computed with history: K - 1 samples for the plain kernel, one tile at tile-aligned positions
 * for the tensor-core form). Allocation and the tap upload come before the clock; `total_ms`
 * (may be NULL) is the wall clock from the first chunk to the last output, `chunks` (may be
 * NULL) the number of chunks. Replaces fir_stream (src/stream.hpp:50-53, src/stream.cu:135-222). */
int rfx_fir_stream(const void* x_iq, int64_t num_samples, const float* taps, int num_taps,
                   const rfx_stream_config* config, void* y_iq, double* total_ms, int* chunks);

/* rfx_fir_stream over host samples stored in `format` (rfx_sample_format): each chunk's stored
 * bytes are uploaded (a half or a quarter of cf32's for ci16 / ci8) and converted by the
 * kernels, with the bits of streaming the host-converted samples. y_iq is cf32. */
int rfx_fir_stream_format(int format, const void* x, int64_t num_samples, const float* taps,
                          int num_taps, const rfx_stream_config* config, void* y_iq,
                          double* total_ms, int* chunks);

/* ---- host-buffer operations (timed like the project's Bench) --------------------------- */

/* Phase timings of a host-buffer call, as the project's BenchResult (src/bench.hpp:17-32). */
typedef struct rfx_bench {
    int warmup;              /* in: untimed passes */
    int runs;                /* in: timed passes (>= 1) */
    double h2d_ms_mean, h2d_ms_std;
    double kernel_ms_mean, kernel_ms_std;
    double d2h_ms_mean, d2h_ms_std;
} rfx_bench;

/* The FIR on host buffers: allocates device memory (setup, untimed), then `runs` passes of
 * upload / compute / download timed with CUDA events. `x_iq`/`y_iq` are host cf32 arrays.
 * `block` is accepted for the project's --block (a multiple of 32, at most 1024) and does
 * not change the result. `bench` may be NULL (one untimed pass).
 * Replaces the FirFn table entries (src/ops.hpp:33-36). */
int rfx_fir_host(int impl, const void* x_iq, int64_t num_samples, const float* taps,
                 int num_taps, int block, void* y_iq, rfx_bench* bench);

/* rfx_fir_host over host samples in `format` (rfx_sample_format): the stored bytes are
 * uploaded and converted on the device by rfx_fir_launch_format; bench->h2d covers those bytes. */
int rfx_fir_host_format(int impl, int format, const void* x, int64_t num_samples,
                        const float* taps, int num_taps, int block, void* y_iq, rfx_bench* bench);

/* The channelizer on host buffers, as above. `z_iq` receives frames * channels cf32.
 * Replaces channelize_cuda (src/ops.hpp:40-41). */
int rfx_channelize_host(int impl, const void* x_iq, int64_t num_samples, const float* taps,
                        int num_taps, int channels, void* z_iq, rfx_bench* bench);

/* rfx_channelize_magnitude_launch on host buffers: `mag` receives frames * channels float32. */
int rfx_channelize_magnitude_host(int impl, const void* x_iq, int64_t num_samples,
                                  const float* taps, int num_taps, int channels, float* mag,
                                  rfx_bench* bench);

/* The channelizer on host samples stored in `format`, with either output (rfx_chan_output):
 * the stored bytes are uploaded; `out` receives frames * channels cf32 or float32. */
int rfx_channelize_host_format(int impl, int format, int output, const void* x,
                               int64_t num_samples, const float* taps, int num_taps,
                               int channels, void* out, rfx_bench* bench);

/* The magnitude on host buffers. Replaces magnitude_cuda (src/ops.hpp:27-29). */
int rfx_magnitude_host(const void* x_iq, int64_t num_samples, float* mag, rfx_bench* bench);

/* ---- tuning --------------------------------------------------------------------------- */

/* The `auto` implementations consult in-process tables filled by the calls below, and apply
 * a built-in rule where an entry is missing (FIR: the tensor core from 32 taps and 2^16
 * samples; channelizer: the tensor core at 64 channels). A batch plan's auto form puts every
 * capture of 2 taps or more on a tensor-core phase; rfx_fir_batch_launch's auto form follows
 * the FIR table beyond 385 taps and takes the tensor core from 160 taps (and 2^16 samples)
 * otherwise. If the environment variable RFX_TUNE_FILE names a file saved by
 * rfx_autotune_save, it is loaded before the first lookup (entries of other GPUs or drivers
 * are skipped). The tuner is this library's own: the project picks kernels by name only
 * (src/main.cpp:156-167), and its plan object for a channelizer is a cuFFT plan. */

/* Times every candidate of `impl` (RFX_FIR_AUTO: the plain kernel and every tensor-core tile
 * shape) for one (num_taps, num_samples) FIR case on the current device, over seeded
 * pseudo-random samples and taps, and stores the fastest for that (taps, length) bucket (powers
 * of two). Allocates scratch buffers; synchronizes. `best_ms` may be NULL. */
int rfx_autotune_fir(int impl, int num_taps, int64_t num_samples, double* best_ms);

/* The same for the channelizer: times the plain and (where it exists) the tensor-core form
 * for `channels` channels, `num_taps` taps, `num_samples` samples, and stores the faster for
 * RFX_CHAN_AUTO plans of that channel count and length bucket. */
int rfx_autotune_channelize(int channels, int num_taps, int64_t num_samples, double* best_ms);

/* Writes / reads the tuned tables as text (one line per entry, keyed by GPU name and driver).
 * rfx_autotune_clear empties them (the built-in rules apply again). */
int rfx_autotune_save(const char* path);
int rfx_autotune_load(const char* path);
int rfx_autotune_clear(void);

#ifdef __cplusplus
}
#endif

#endif /* RFX_H */
