// Plain channelizer: FP32 polyphase branch sums, then cuFFT's batched inverse transform in
// place — the structure of the project's channelize_device (src/channelize.cu:56-72).
//
//   u[t][m] = sum_p h[pM + m] x[tM - pM - m]          (x[i < 0] = 0)
//   z[t][k] = sum_m u[t][m] e^{+2 pi i k m / M}        (cuFFT inverse, unnormalized)
//
// The branch sums use the project's arithmetic (src/channelize.cu:35-46): one fused
// multiply-add per tap, l = m, m + M, ... ascending from +0, skipping the terms before the start
// of the input, so u is bit-identical to its kernel's. The project runs one thread per (frame,
// branch), which reads every sample once per tap of its branch (32 times at 32 taps per branch)
// through the caches. Here the frames of one branch are a FIR over the decimated sequence
// s_d = x[dM - m] with taps g_p = h[pM + m], and consecutive threads take consecutive branches,
// so every sample and tap load of a warp is one coalesced 256-byte row; the I/Q pair is one
// packed f32x2 fused multiply-add. Two forms:
//  - chan_branch_ring_kernel (8, 16, 24 or 32 taps in every branch): a thread walks one branch
//    through a segment of frames keeping the window of its current 8 frames in registers, so
//    each sample is loaded once (2^26 samples, 1024 channels, 32 taps per branch: 187 us under
//    the profiler, 84 % of the HBM copy rate, against 350 us for the form below);
//  - chan_branch_kernel (any tap count): a thread computes R = 8 consecutive frames of one
//    branch with two alternating 8-sample register blocks, so each sample is loaded
//    (R + P - 1) / R times instead of P times.
// Frame groups whose terms fall before the input, and the last group (past its end), take a
// path that tests every term.
#include "chan_plain.cuh"
#include "ptx.cuh"

#include <cuda_runtime.h>
#include <cufft.h>

namespace rfx {

namespace {
constexpr int kBranchThreads = 256;
constexpr int kR = 8;   // frames per thread

// Taps p0 + q (q < nq) of one branch: acc[i] += g_p s_{t0 + i - p}, with cur[i] = s_{t0 - 8g + i}
// and nxt[i] = s_{t0 - 8(g+1) + i} for p0 = 8 g. Guarded: only terms whose sample index is >= 0.
template <bool kGuard>
__device__ __forceinline__ void taps_block(f32x2 (&acc)[kR], const f32x2 (&cur)[kR],
                                           const f32x2 (&nxt)[kR], const float* tcol,
                                           int tstride, int p0, int nq, long long t0,
                                           int first_valid_d)
{
#pragma unroll
    for (int q = 0; q < kR; ++q) {
        if (q < nq) {
            const float hv = tcol[(p0 + q) * tstride];
            const f32x2 h2 = pack2(hv, hv);
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                const f32x2 v = i >= q ? cur[i - q] : nxt[kR + i - q];
                if (!kGuard || t0 + i - (p0 + q) >= first_valid_d) {
                    acc[i] = fma2(h2, v, acc[i]);
                }
            }
        }
    }
}

// Sample s of x in format kFmt (0 cf32; 1 ci16, 2 ci8: components converted as the project's
// SigMF reader converts them, src/io.cpp:110-148, so the sums are those of the converted input).
template <int kFmt>
__device__ __forceinline__ f32x2 load_sample(const void* __restrict__ x, long long s)
{
    if constexpr (kFmt == 0) {
        const float2 w = __ldg(static_cast<const float2*>(x) + s);
        return pack2(w.x, w.y);
    } else if constexpr (kFmt == 1) {
        const short2 w = __ldg(static_cast<const short2*>(x) + s);
        return pack2(static_cast<float>(w.x) * (1.0f / 32768.0f),
                     static_cast<float>(w.y) * (1.0f / 32768.0f));
    } else {
        const char2 w = __ldg(static_cast<const char2*>(x) + s);
        return pack2(static_cast<float>(w.x) * (1.0f / 128.0f),
                     static_cast<float>(w.y) * (1.0f / 128.0f));
    }
}

template <bool kGuard, int kFmt>
__device__ __forceinline__ void load_block(f32x2 (&blk)[kR], const void* __restrict__ x,
                                           long long n, int channels, int m, long long d0)
{
#pragma unroll
    for (int i = 0; i < kR; ++i) {
        const long long s = (d0 + i) * channels - m;
        f32x2 v = 0ull;
        if (!kGuard || (s >= 0 && s < n)) {
            v = load_sample<kFmt>(x, s);
        }
        blk[i] = v;
    }
}

template <bool kGuard, int kFmt>
__device__ __forceinline__ void branch_frames(f32x2 (&acc)[kR], const void* __restrict__ x,
                                              const float* tcol, int tstride, long long n,
                                              int channels, int m, int P, long long t0)
{
    const int first_valid_d = m > 0 ? 1 : 0;   // x[dM - m] >= 0 from this d on
    const int groups = P / kR;
    const int rem = P - groups * kR;
    f32x2 a[kR];
    f32x2 b[kR];
    load_block<kGuard, kFmt>(a, x, n, channels, m, t0);
    int g = 0;
    for (; g + 2 <= groups; g += 2) {
        load_block<kGuard, kFmt>(b, x, n, channels, m, t0 - kR * (g + 1));
        taps_block<kGuard>(acc, a, b, tcol, tstride, kR * g, kR, t0, first_valid_d);
        load_block<kGuard, kFmt>(a, x, n, channels, m, t0 - kR * (g + 2));
        taps_block<kGuard>(acc, b, a, tcol, tstride, kR * (g + 1), kR, t0, first_valid_d);
    }
    if (g < groups) {
        load_block<kGuard, kFmt>(b, x, n, channels, m, t0 - kR * (g + 1));
        taps_block<kGuard>(acc, a, b, tcol, tstride, kR * g, kR, t0, first_valid_d);
        if (rem > 0) {
            load_block<kGuard, kFmt>(a, x, n, channels, m, t0 - kR * (g + 2));
            taps_block<kGuard>(acc, b, a, tcol, tstride, kR * (g + 1), rem, t0,
                               first_valid_d);
        }
    } else if (rem > 0) {
        load_block<kGuard, kFmt>(b, x, n, channels, m, t0 - kR * (g + 1));
        taps_block<kGuard>(acc, a, b, tcol, tstride, kR * g, rem, t0, first_valid_d);
    }
}
}  // namespace

// Block: `width` consecutive branches x (256 / width) frame groups of kR frames per step, over
// kGroupSteps consecutive steps. With kSmemTaps the block's taps (max_p x width) are staged in
// shared memory once, and its consecutive frame groups reuse each other's samples through L1
// (measured at 2^26 samples, 1024 channels, 32 taps per branch: 490 us against 533 us reading
// taps through the caches one frame group per block). Groups with t0 < guard_frames or
// reaching past the last frame test every load and term.
constexpr int kGroupSteps = 16;

template <int kFmt, bool kSmemTaps>
__global__ void __launch_bounds__(kBranchThreads)
chan_branch_kernel(const void* __restrict__ x, const float* __restrict__ taps,
                   float2* __restrict__ u, long long n, long long frames, int channels,
                   int num_taps, int width, int guard_frames)
{
    extern __shared__ float taps_s[];   // [p][j]: tap p of branch blockIdx.y * width + j
    const int j = static_cast<int>(threadIdx.x) % width;
    const int m = static_cast<int>(blockIdx.y) * width + j;
    if (kSmemTaps) {
        const int max_p = (num_taps + channels - 1) / channels;
        for (int i = threadIdx.x; i < max_p * width; i += kBranchThreads) {
            const int p = i / width;
            const int jj = i - p * width;
            const int mm = static_cast<int>(blockIdx.y) * width + jj;
            const long long l = static_cast<long long>(p) * channels + mm;
            taps_s[i] = (mm < channels && l < num_taps) ? __ldg(taps + l) : 0.0f;
        }
        __syncthreads();
    }
    if (m >= channels) {
        return;
    }
    // Taps of branch m: l = pM + m < num_taps; read from column j of the staged table, or from
    // global memory at stride `channels`.
    const int P = m < num_taps ? (num_taps - m + channels - 1) / channels : 0;
    const float* tcol = kSmemTaps ? taps_s + j : taps + m;
    const int tstride = kSmemTaps ? width : channels;
    const int steps = kSmemTaps ? kGroupSteps : 1;
    for (int it = 0; it < steps; ++it) {
        const long long group = (static_cast<long long>(blockIdx.x) * steps + it) *
                                    (kBranchThreads / width) + threadIdx.x / width;
        const long long t0 = group * kR;
        if (t0 >= frames) {
            return;
        }
        f32x2 acc[kR];
#pragma unroll
        for (int i = 0; i < kR; ++i) {
            acc[i] = 0ull;
        }
        if (t0 < guard_frames || t0 + kR > frames) {
            branch_frames<true, kFmt>(acc, x, tcol, tstride, n, channels, m, P, t0);
        } else {
            branch_frames<false, kFmt>(acc, x, tcol, tstride, n, channels, m, P, t0);
        }
#pragma unroll
        for (int i = 0; i < kR; ++i) {
            if (t0 + i < frames) {
                u[(t0 + i) * channels + m] = unpack2(acc[i]);
            }
        }
    }
}

// Register-ring form, for filters of exactly 8, 16, 24 or 32 taps in every branch (num_taps =
// P * channels; cf32 and ci16 input). A thread owns one branch m and one segment of
// consecutive frames, which it walks in steps of kR = 8 frames. The samples of its branch for
// the current step and the P / 8 steps before it (a step's window: P + 8 decimated samples)
// stay in registers as P / 8 + 1 blocks of eight, so every sample is loaded once per segment
// instead of once per tap group, and the branch's taps stay in registers too. The next blocks
// stream in by per-thread asynchronous copies, kRingStages steps ahead, into the thread's own
// slots of a shared-memory stage ring (a warp's copies and reads of one block row are 256
// contiguous bytes). Terms are summed in branch_frames' order: taps ascending from +0, one
// fused multiply-add each; steps whose terms reach before the input (t0 < guard_frames) take
// branch_frames' tested path. Every branch having all P taps, the tap loop has no per-branch
// test (measured: a per-tap test of the branch's tap count doubled the instructions issued).
constexpr int kRingThreads = 128;
constexpr int kRingStages = 4;

template <int kFmt>
__device__ __forceinline__ f32x2 ring_lds(uint32_t addr)
{
    if constexpr (kFmt == 0) {
        return lds64(addr);
    } else {
        uint32_t w;
        asm volatile("ld.shared.u32 %0, [%1];" : "=r"(w) : "r"(addr));
        return pack2(static_cast<float>(static_cast<int>(w << 16) >> 16) * (1.0f / 32768.0f),
                     static_cast<float>(static_cast<int>(w) >> 16) * (1.0f / 32768.0f));
    }
}

template <int kPG, int kFmt>
__global__ void __launch_bounds__(kRingThreads, 3)
chan_branch_ring_kernel(const void* __restrict__ x, const float* __restrict__ taps,
                        float2* __restrict__ u, long long n, long long frames, int channels,
                        int width, long long seg_frames, int guard_frames)
{
    constexpr int kN = kPG + 1;                  // register blocks
    constexpr int kP = kR * kPG;                 // taps per branch
    constexpr int kSb = kFmt == 0 ? 8 : 4;       // bytes per stored sample
    constexpr uint32_t kStageBytes = kR * kRingThreads * kSb;
    __shared__ __align__(16) unsigned char stage[kRingStages * kStageBytes];
    const int tid = static_cast<int>(threadIdx.x);
    const int j = tid % width;
    const int m = static_cast<int>(blockIdx.y) * width + j;
    const long long seg = static_cast<long long>(blockIdx.x) * (kRingThreads / width) + tid / width;
    const long long f0 = seg * seg_frames;
    if (m >= channels || f0 >= frames) {
        return;
    }
    const long long f1 = f0 + seg_frames < frames ? f0 + seg_frames : frames;
    float g[kP];
#pragma unroll
    for (int p = 0; p < kP; ++p) {
        g[p] = __ldg(taps + static_cast<long long>(p) * channels + m);
    }
    long long t0 = f0;
    for (; t0 < f1 && t0 < guard_frames; t0 += kR) {
        f32x2 acc[kR];
#pragma unroll
        for (int i = 0; i < kR; ++i) {
            acc[i] = 0ull;
        }
        branch_frames<true, kFmt>(acc, x, taps + m, channels, n, channels, m, kP, t0);
#pragma unroll
        for (int i = 0; i < kR; ++i) {
            if (t0 + i < f1) {
                u[(t0 + i) * channels + m] = unpack2(acc[i]);
            }
        }
    }
    if (t0 >= f1) {
        return;
    }
    // Ring slot k % kN holds block B(t0 + 8k) (decimated samples t0 + 8k .. + 7) during step k;
    // the blocks before step 0 go to slots kN - q, q = 1 .. kPG (all at indices >= 8 M - m).
    f32x2 R[kN][kR];
#pragma unroll
    for (int q = 1; q <= kPG; ++q) {
#pragma unroll
        for (int i = 0; i < kR; ++i) {
            R[kN - q][i] = load_sample<kFmt>(x, (t0 - kR * q + i) * channels - m);
        }
    }
    // Sample d of the branch is at byte (d M - m) kSb of x: consecutive d are `row` bytes apart.
    const long long row = static_cast<long long>(channels) * kSb;
    // Slot (stage s, sample i) of this thread: stage + s * kStageBytes + (i * 128 + tid) * kSb.
    const uint32_t sbase = smem_u32(stage) + static_cast<uint32_t>(tid * kSb);
    const long long nb = (f1 - t0 + kR - 1) / kR;
    // The next block to copy: its first sample's address and how many of its samples lie in
    // the segment.
    const char* src = static_cast<const char*>(x) + (t0 * channels - m) * kSb;
    long long src_left = f1 - t0;
    uint32_t src_stage = 0;
    auto issue = [&]() {
        const uint32_t dst = sbase + src_stage * kStageBytes;
        if (src_left >= kR) {
            const char* s = src;
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                cp_async<kSb>(dst + static_cast<uint32_t>(i * kRingThreads * kSb), s, kSb);
                s += row;
            }
        } else {
            const char* s = src;
#pragma unroll
            for (int i = 0; i < kR; ++i) {
                const bool ok = i < src_left;
                cp_async<kSb>(dst + static_cast<uint32_t>(i * kRingThreads * kSb), ok ? s : src,
                              ok ? kSb : 0);
                s += row;
            }
        }
        cp_async_commit();
        src += kR * row;
        src_left -= kR;
        src_stage = src_stage + 1 == kRingStages ? 0 : src_stage + 1;
    };
#pragma unroll
    for (int s = 0; s < kRingStages - 1; ++s) {
        issue();
    }
    float2* dst = u + t0 * channels + m;
    long long dst_left = f1 - t0;
    uint32_t read_stage = 0;
    for (long long k0 = 0; k0 < nb; k0 += kN) {
#pragma unroll
        for (int rot = 0; rot < kN; ++rot) {
            if (k0 + rot < nb) {
                // Refills the stage read in the step before with the block kRingStages - 1
                // steps ahead, then waits for this step's block.
                issue();
                cp_async_wait<kRingStages - 1>();
                const uint32_t rs = sbase + read_stage * kStageBytes;
                read_stage = read_stage + 1 == kRingStages ? 0 : read_stage + 1;
#pragma unroll
                for (int i = 0; i < kR; ++i) {
                    R[rot][i] = ring_lds<kFmt>(rs + static_cast<uint32_t>(i * kRingThreads * kSb));
                }
                f32x2 acc[kR];
#pragma unroll
                for (int i = 0; i < kR; ++i) {
                    acc[i] = 0ull;
                }
                // Tap group gq: cur = B(T - 8 gq), nxt = B(T - 8 gq - 8), T = t0 + 8 k.
#pragma unroll
                for (int gq = 0; gq < kPG; ++gq) {
                    const int cs = (rot - gq + 2 * kN) % kN;
                    const int ns = (rot - gq - 1 + 2 * kN) % kN;
#pragma unroll
                    for (int q = 0; q < kR; ++q) {
                        const f32x2 h2 = pack2(g[kR * gq + q], g[kR * gq + q]);
#pragma unroll
                        for (int i = 0; i < kR; ++i) {
                            acc[i] = fma2(h2, i >= q ? R[cs][i - q] : R[ns][kR + i - q], acc[i]);
                        }
                    }
                }
                if (dst_left >= kR) {
                    float2* o = dst;
#pragma unroll
                    for (int i = 0; i < kR; ++i) {
                        *o = unpack2(acc[i]);
                        o += channels;
                    }
                } else {
                    float2* o = dst;
#pragma unroll
                    for (int i = 0; i < kR; ++i) {
                        if (i < dst_left) {
                            *o = unpack2(acc[i]);
                        }
                        o += channels;
                    }
                }
                dst += static_cast<long long>(kR) * channels;
                dst_left -= kR;
            }
        }
    }
    cp_async_wait<0>();
}

static cudaError_t ring_launch(const void* x, const float* taps, float2* u, long long n,
                               long long frames, int channels, int per_branch,
                               cudaStream_t stream, int format)
{
    const void* fn = nullptr;
    switch (per_branch / kR * 2 + format) {
    case 2: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<1, 0>); break;
    case 3: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<1, 1>); break;
    case 4: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<2, 0>); break;
    case 5: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<2, 1>); break;
    case 6: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<3, 0>); break;
    case 7: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<3, 1>); break;
    case 8: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<4, 0>); break;
    case 9: fn = reinterpret_cast<const void*>(chan_branch_ring_kernel<4, 1>); break;
    default: return cudaErrorInvalidValue;
    }
    int device = 0;
    int sms = 0;
    int occ = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) !=
            cudaSuccess ||
        (err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kRingThreads, 0)) !=
            cudaSuccess) {
        return err;
    }
    // Branches per block: all (up to 128), or the power of two >= channels with several
    // segments per block. One wave of blocks: segments of equal length cover the frames.
    int w = 32;
    while (w < channels && w < kRingThreads) {
        w *= 2;
    }
    const int per_block = kRingThreads / w;
    const long long gy = (channels + w - 1) / w;
    const long long capacity = static_cast<long long>(sms) * (occ > 0 ? occ : 1);
    const long long bx_target = capacity / gy > 0 ? capacity / gy : 1;
    const long long segs_target = bx_target * per_block;
    long long seg_frames = (frames + segs_target - 1) / segs_target;
    seg_frames = (seg_frames + kR - 1) / kR * kR;
    if (seg_frames < 8 * kR) {
        seg_frames = 8 * kR;
    }
    const long long segs = (frames + seg_frames - 1) / seg_frames;
    const long long bx = (segs + per_block - 1) / per_block;
    if (bx > 0x7FFFFFFFLL || gy > 65535) {
        return cudaErrorInvalidConfiguration;
    }
    int guard_frames = kR * (per_branch / kR + 1);
    const dim3 grid(static_cast<unsigned>(bx), static_cast<unsigned>(gy));
    void* args[] = {&x, &taps, &u, &n, &frames, &channels, &w, &seg_frames, &guard_frames};
    err = cudaLaunchKernel(fn, grid, dim3(kRingThreads), args, 0, stream);
    if (err != cudaSuccess) {
        return err;
    }
    return cudaGetLastError();
}

cudaError_t chan_branch_launch(const void* x, const float* taps, void* u, long long frames,
                               int channels, int num_taps, cudaStream_t stream, int format)
{
    if (frames == 0 || channels < 1) {
        return cudaSuccess;
    }
    {
        const long long n = (frames - 1) * static_cast<long long>(channels) + 1;
        const int per_branch = num_taps / channels;
        if (format <= 1 && num_taps % channels == 0 && per_branch % kR == 0 &&
            per_branch >= kR && per_branch <= 4 * kR) {
            return ring_launch(x, taps, static_cast<float2*>(u), n, frames, channels, per_branch,
                               stream, format);
        }
    }
    // The newest sample any frame reads is the last frame's x[(frames - 1) M], which lies in the
    // input: loads are bounded by that index.
    const long long n = (frames - 1) * static_cast<long long>(channels) + 1;
    // Branches per block: the power of two >= channels, between one warp and the whole block.
    int w = 32;
    while (w < channels && w < kBranchThreads) {
        w *= 2;
    }
    const long long groups = (frames + kR - 1) / kR;
    const int per_block = kBranchThreads / w;
    const long long gy = (channels + w - 1) / w;
    // Frame groups before this one load samples before the input (the lowest sample block a
    // group loads starts kR * ceil(P / kR) frames back): they take the tested path.
    const int max_p = (num_taps + channels - 1) / channels;
    const int guard_frames = kR * ((max_p + kR - 1) / kR + 1);
    const size_t smem_bytes = static_cast<size_t>(max_p) * w * sizeof(float);
    int device = 0;
    int optin = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess ||
        (err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device)) !=
            cudaSuccess) {
        return err;
    }
    const bool staged = smem_bytes <= static_cast<size_t>(optin);
    const long long steps = staged ? kGroupSteps : 1;
    const long long gx = (groups + per_block * steps - 1) / (per_block * steps);
    if (gx > 0x7FFFFFFFLL || gy > 65535) {
        return cudaErrorInvalidConfiguration;
    }
    const dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
    float2* uo = static_cast<float2*>(u);
    auto run = [&](auto kernel, size_t bytes) -> cudaError_t {
        if (bytes > 48 * 1024) {
            const cudaError_t e = cudaFuncSetAttribute(
                kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
            if (e != cudaSuccess) {
                return e;
            }
        }
        kernel<<<grid, kBranchThreads, bytes, stream>>>(x, taps, uo, n, frames, channels,
                                                       num_taps, w, guard_frames);
        return cudaSuccess;
    };
    switch (format * 2 + (staged ? 1 : 0)) {
    case 0: err = run(chan_branch_kernel<0, false>, 0); break;
    case 1: err = run(chan_branch_kernel<0, true>, smem_bytes); break;
    case 2: err = run(chan_branch_kernel<1, false>, 0); break;
    case 3: err = run(chan_branch_kernel<1, true>, smem_bytes); break;
    case 4: err = run(chan_branch_kernel<2, false>, 0); break;
    case 5: err = run(chan_branch_kernel<2, true>, smem_bytes); break;
    default: return cudaErrorInvalidValue;
    }
    if (err != cudaSuccess) {
        return err;
    }
    return cudaGetLastError();
}

}  // namespace rfx
