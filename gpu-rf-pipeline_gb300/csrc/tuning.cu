// The tuned-configuration tables behind the `auto` implementations.
//
// * FIR: which implementation RFX_FIR_AUTO runs and which tile shape the tensor-core FIR uses,
//   per (tap-count bucket, length bucket). rfx_fir_batch_launch's auto form places each capture
//   by the same table, so tuning a capture's (taps, length) bucket tunes the batch's partition.
// * Channelizer: which implementation RFX_CHAN_AUTO plans use, per (channel count, length
//   bucket).
//
// Entries come from timing the candidates on the current device over seeded pseudo-random
// inputs (rfx_autotune_fir, rfx_autotune_channelize); a lookup that finds none applies the
// built-in rule. The tables are saved and loaded as text keyed by GPU name and driver version
// (rfx_autotune_save / rfx_autotune_load); the file named by the environment variable
// RFX_TUNE_FILE, if set, is loaded automatically before the first lookup.
#include "rfx.h"
#include "tuning.hpp"
#include "chan_tc.cuh"
#include "chan_wide.cuh"
#include "fir_plain.cuh"
#include "fir_tc.cuh"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

namespace rfx {

namespace {

struct FirEntry {
    int impl;
    TcConfig config;
    double ms;
};

struct ChanEntry {
    int impl;
    double ms;
};

// Buckets: taps by power of two (1, 2-3, 4-7, ...), lengths by power of two.
int bucket(long long v)
{
    int b = 0;
    while (v > 1) {
        v >>= 1;
        ++b;
    }
    return b;
}

std::mutex g_mutex;
std::map<std::pair<int, int>, FirEntry> g_fir;    // (taps bucket, length bucket)
std::map<std::pair<int, int>, ChanEntry> g_chan;  // (channels, length bucket)

int load_table(const char* path);  // below; takes g_mutex

// Loads $RFX_TUNE_FILE once, before the first lookup (a missing file is not an error).
void load_environment_table()
{
    static std::once_flag once;
    std::call_once(once, [] {
        const char* path = std::getenv("RFX_TUNE_FILE");
        if (path != nullptr && path[0] != '\0') {
            load_table(path);
        }
    });
}

bool lookup_fir(int num_taps, long long n, FirEntry* out)
{
    load_environment_table();
    std::lock_guard<std::mutex> lock(g_mutex);
    const auto it = g_fir.find({bucket(num_taps), bucket(n)});
    if (it == g_fir.end()) {
        return false;
    }
    *out = it->second;
    return true;
}

bool lookup_chan(int channels, long long n, ChanEntry* out)
{
    load_environment_table();
    std::lock_guard<std::mutex> lock(g_mutex);
    const auto it = g_chan.find({channels, bucket(n)});
    if (it == g_chan.end()) {
        return false;
    }
    *out = it->second;
    return true;
}

std::string device_key()
{
    int dev = 0;
    cudaDeviceProp prop{};
    int driver = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return "unknown";
    }
    cudaDriverGetVersion(&driver);
    std::string name = prop.name;
    for (char& ch : name) {
        if (ch == ' ') {
            ch = '_';
        }
    }
    return name + "/" + std::to_string(driver);
}

// Text format, one entry per line:
//   fir  <device key> <taps bucket> <length bucket> <impl> <tile blocks> <stages> <ms>
//   chan <device key> <channels> <length bucket> <impl> <ms>
int load_table(const char* path)
{
    FILE* f = std::fopen(path, "r");
    if (f == nullptr) {
        return RFX_ERR_INVALID;
    }
    const std::string key = device_key();
    char line[512];
    std::lock_guard<std::mutex> lock(g_mutex);
    while (std::fgets(line, sizeof(line), f) != nullptr) {
        char kind[8];
        char dev[256];
        int a, b, impl, blocks, stages;
        double ms;
        if (std::sscanf(line, "%7s %255s", kind, dev) != 2 || key != dev) {
            continue;
        }
        if (std::strcmp(kind, "fir") == 0 &&
            std::sscanf(line, "%*s %*s %d %d %d %d %d %lf", &a, &b, &impl, &blocks, &stages,
                        &ms) == 6 &&
            (impl == RFX_FIR_PLAIN || impl == RFX_FIR_TC)) {
            g_fir[{a, b}] = FirEntry{impl, TcConfig{blocks, stages}, ms};
        } else if (std::strcmp(kind, "chan") == 0 &&
                   std::sscanf(line, "%*s %*s %d %d %d %lf", &a, &b, &impl, &ms) == 4 &&
                   (impl == RFX_CHAN_PLAIN || impl == RFX_CHAN_TC)) {
            g_chan[{a, b}] = ChanEntry{impl, ms};
        }
    }
    std::fclose(f);
    return RFX_OK;
}

// Seeded pseudo-random values in [-scale, scale): the tuner's inputs (timing on zeros could
// flatter data-dependent paths such as the tensor-core FIR's per-tile scale search).
__global__ void fill_kernel(float* p, long long count, unsigned seed, float scale)
{
    const long long stride = static_cast<long long>(gridDim.x) * blockDim.x;
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < count;
         i += stride) {
        unsigned h = static_cast<unsigned>(i) * 0x9E3779B1u ^ seed;
        h ^= h >> 16;
        h *= 0x85EBCA6Bu;
        h ^= h >> 13;
        h *= 0xC2B2AE35u;
        h ^= h >> 16;
        p[i] = scale * (static_cast<float>(h >> 8) * (1.0f / 8388608.0f) - 1.0f);
    }
}

cudaError_t fill(void* p, long long floats, unsigned seed, float scale)
{
    fill_kernel<<<1024, 256>>>(static_cast<float*>(p), floats, seed, scale);
    return cudaGetLastError();
}

// Scratch inputs for one tuning call: x and an output of `samples` cf32, `taps` floats.
struct Scratch {
    void* x = nullptr;
    void* y = nullptr;
    float* h = nullptr;

    cudaError_t make(long long samples, long long out_samples, int taps)
    {
        cudaError_t err = cudaMalloc(&x, static_cast<size_t>(samples) * 8);
        if (err == cudaSuccess) {
            err = cudaMalloc(&y, static_cast<size_t>(out_samples) * 8);
        }
        if (err == cudaSuccess) {
            err = cudaMalloc(&h, sizeof(float) * taps);
        }
        if (err == cudaSuccess) {
            err = fill(x, 2 * samples, 0x5eedu, 1.0f);
        }
        if (err == cudaSuccess) {
            err = fill(h, taps, 0x7a95u, 1.0f / static_cast<float>(taps));
        }
        if (err == cudaSuccess) {
            err = cudaDeviceSynchronize();
        }
        return err;
    }

    ~Scratch()
    {
        cudaFree(x);
        cudaFree(y);
        cudaFree(h);
    }
};

// Best of five timed runs after one untimed run; a negative value when `run` fails.
template <class Run>
double best_ms(Run run)
{
    if (run() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        return -1.0;
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        cudaEventRecord(a, nullptr);
        run();
        cudaEventRecord(b, nullptr);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        best = ms < best ? ms : best;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return best;
}

}  // namespace

// Built-in rule before tuning: the tensor-core form once the filter is long enough for FP32
// FMA throughput to bound the plain kernel and the input fills the GPU; the plain kernel
// otherwise. Measured on GB300 at 2^24 samples: the plain kernel is HBM-bound up to about 24
// taps (42-49 us) and FMA-bound beyond (79 us at 63 taps, 149 us at 129); the resident-window
// tensor-core form takes 48-58 us from 2 to 129 taps, 68 us at 255 and 82 us at 385; the
// long-filter form 120 us at 511 taps and 141 us at 1025.
int tuned_fir_impl(int num_taps, long long n)
{
    FirEntry e;
    if (lookup_fir(num_taps, n, &e)) {
        return e.impl;
    }
    constexpr int kTcMinTaps = 32;
    constexpr long long kTcMinSamples = 1LL << 16;
    return num_taps >= kTcMinTaps && n >= kTcMinSamples && fir_tc_supported(num_taps)
               ? RFX_FIR_TC
               : RFX_FIR_PLAIN;
}

// Where rfx_fir_batch_launch places a capture. Its tensor-core kernel is the long-filter form
// (fir_batch.cu), whose tiles cost about the same whatever the filter, so short filters stay on
// the plain tiles: the tensor core from 160 taps (plain and the long-filter form meet near 130),
// or where a tuned entry for a filter beyond the resident-window form's range says so.
int tuned_fir_batch_launch_impl(int num_taps, long long n)
{
    FirEntry e;
    if (!fir_tcw_supported(num_taps) && lookup_fir(num_taps, n, &e)) {
        return e.impl;
    }
    constexpr int kTcMinTaps = 160;
    constexpr long long kTcMinSamples = 1LL << 16;
    return num_taps >= kTcMinTaps && n >= kTcMinSamples && fir_tc_supported(num_taps)
               ? RFX_FIR_TC
               : RFX_FIR_PLAIN;
}

// Where a batch plan places a capture: a tensor-core phase for every filter of two taps or more
// that one takes (its window phase up to 385 taps, its long-filter phase beyond), at any length:
// a plan launches once for the whole batch, so a short capture is no reason for the plain tiles.
// Measured on the 256-capture workload (batch plans of each tap count alone): a window tile of
// 6144 outputs costs 2.9-3.6 SM-us at 31-127 taps, 4.1 at 255, a long-filter tile of 12288
// outputs 16.5-18.6 SM-us at 511-1025, against 2304-output plain tiles of 1.7 SM-us at 31 taps
// and 12.6-24.7 at 511-1025 (per output the tensor-core tiles cost less at every tap count);
// putting the short captures of long filters on the plain tiles instead made the whole batch
// 4 % slower.
int tuned_fir_batch_impl(int num_taps, long long n)
{
    (void)n;
    return num_taps >= 2 && (fir_tcw_supported(num_taps) || fir_batch_supported(num_taps))
               ? RFX_FIR_TC
               : RFX_FIR_PLAIN;
}

TcConfig tuned_fir_tc_config(int num_taps, long long n)
{
    FirEntry e;
    if (lookup_fir(num_taps, n, &e) && e.impl == RFX_FIR_TC) {
        return e.config;
    }
    // The resident-window form where it applies (one copy of each window, no scan slices).
    return fir_tcw_supported(num_taps) ? TcConfig{kTcWindowTile, 4} : TcConfig{96, 6};
}

// Built-in rule: the fused tensor-core form at 64 channels (one HBM pass against the plain
// form's two); cuFFT's plain form elsewhere, including 1024 channels, where the branch-sum
// kernel + cuFFT measured faster than the factored tensor-core DFT on GB300.
int tuned_chan_impl(int channels, long long n)
{
    ChanEntry e;
    if (lookup_chan(channels, n, &e)) {
        return e.impl;
    }
    return chan_tc_supported(channels, 1) ? RFX_CHAN_TC : RFX_CHAN_PLAIN;
}

}  // namespace rfx

extern "C" int rfx_autotune_fir(int impl, int num_taps, int64_t num_samples, double* best_out)
{
    using namespace rfx;
    if (num_taps < 1 || num_taps > kMaxTaps || num_samples < 1 || num_samples > INT32_MAX) {
        return RFX_ERR_INVALID;
    }
    Scratch s;
    if (s.make(num_samples, num_samples, num_taps) != cudaSuccess) {
        cudaGetLastError();
        return RFX_ERR_CUDA;
    }
    struct Candidate {
        int impl;
        TcConfig config;
    };
    std::vector<Candidate> candidates;
    if (impl == RFX_FIR_PLAIN || impl == RFX_FIR_AUTO) {
        candidates.push_back({RFX_FIR_PLAIN, TcConfig{0, 0}});
    }
    if ((impl == RFX_FIR_TC || impl == RFX_FIR_AUTO) && fir_tc_supported(num_taps)) {
        for (int st : {2, 4, 6}) {
            candidates.push_back({RFX_FIR_TC, TcConfig{96, st}});
        }
        for (int st : {2, 4, 6}) {
            candidates.push_back({RFX_FIR_TC, TcConfig{kTcPairTile, st}});
        }
        if (fir_tcw_supported(num_taps)) {
            candidates.push_back({RFX_FIR_TC, TcConfig{kTcWindowTile, 4}});
        }
    }
    FirEntry best{RFX_FIR_PLAIN, TcConfig{96, 6}, 1e30};
    for (const Candidate& c : candidates) {
        const double ms = best_ms([&]() {
            return c.impl == RFX_FIR_TC
                       ? fir_tc_launch(s.x, s.h, s.y, num_samples, num_taps, c.config, nullptr)
                       : fir_plain_launch(s.x, s.h, s.y, num_samples, num_taps, nullptr);
        });
        if (ms >= 0 && ms < best.ms) {
            best = FirEntry{c.impl, c.config, ms};
        }
    }
    if (best.ms >= 1e29) {
        return RFX_ERR_CUDA;
    }
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        g_fir[{bucket(num_taps), bucket(num_samples)}] = best;
    }
    if (best_out != nullptr) {
        *best_out = best.ms;
    }
    return RFX_OK;
}

extern "C" int rfx_autotune_channelize(int channels, int num_taps, int64_t num_samples,
                                       double* best_out)
{
    using namespace rfx;
    if (channels < 1 || num_taps < 1 || num_samples < channels || num_samples > INT32_MAX) {
        return RFX_ERR_INVALID;
    }
    const long long frames = rfx_channelize_frames(num_samples, channels);
    Scratch s;
    if (s.make(num_samples, frames * channels, num_taps) != cudaSuccess) {
        cudaGetLastError();
        return RFX_ERR_CUDA;
    }
    ChanEntry best{RFX_CHAN_PLAIN, 1e30};
    for (int impl : {RFX_CHAN_PLAIN, RFX_CHAN_TC}) {
        rfx_chan_plan* plan = nullptr;
        if (rfx_chan_plan_create(impl, channels, num_samples, &plan) != RFX_OK) {
            continue;  // e.g. no tensor-core form at this channel count
        }
        const double ms = best_ms([&]() {
            return rfx_channelize_launch(plan, s.x, s.h, s.y, num_samples, num_taps, nullptr) ==
                           RFX_OK
                       ? cudaSuccess
                       : cudaErrorUnknown;
        });
        rfx_chan_plan_destroy(plan);
        if (ms >= 0 && ms < best.ms) {
            best = ChanEntry{impl, ms};
        }
    }
    if (best.ms >= 1e29) {
        return RFX_ERR_CUDA;
    }
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        g_chan[{channels, bucket(num_samples)}] = best;
    }
    if (best_out != nullptr) {
        *best_out = best.ms;
    }
    return RFX_OK;
}

extern "C" int rfx_autotune_save(const char* path)
{
    using namespace rfx;
    if (path == nullptr) {
        return RFX_ERR_INVALID;
    }
    FILE* f = std::fopen(path, "w");
    if (f == nullptr) {
        return RFX_ERR_INVALID;
    }
    const std::string key = device_key();
    std::lock_guard<std::mutex> lock(g_mutex);
    for (const auto& kv : g_fir) {
        std::fprintf(f, "fir %s %d %d %d %d %d %.6f\n", key.c_str(), kv.first.first,
                     kv.first.second, kv.second.impl, kv.second.config.tile_blocks,
                     kv.second.config.stages, kv.second.ms);
    }
    for (const auto& kv : g_chan) {
        std::fprintf(f, "chan %s %d %d %d %.6f\n", key.c_str(), kv.first.first, kv.first.second,
                     kv.second.impl, kv.second.ms);
    }
    std::fclose(f);
    return RFX_OK;
}

extern "C" int rfx_autotune_load(const char* path)
{
    return path == nullptr ? RFX_ERR_INVALID : rfx::load_table(path);
}

extern "C" int rfx_autotune_clear(void)
{
    std::lock_guard<std::mutex> lock(rfx::g_mutex);
    rfx::g_fir.clear();
    rfx::g_chan.clear();
    return RFX_OK;
}
