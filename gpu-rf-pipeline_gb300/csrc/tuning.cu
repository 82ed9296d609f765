// The tuned-configuration table: which FIR implementation RFX_FIR_AUTO runs and which tile
// shape the tensor-core FIR uses, per (tap-count bucket, length bucket). Filled by timing the
// candidates on the current device (rfx_autotune_fir), persisted as text keyed by GPU name
// and driver version (rfx_autotune_save / rfx_autotune_load).
#include "rfx.h"
#include "tuning.hpp"
#include "fir_plain.cuh"
#include "fir_tc.cuh"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

namespace rfx {

namespace {

struct Entry {
    int impl;
    TcConfig config;
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
std::map<std::pair<int, int>, Entry> g_table;

bool lookup(int num_taps, long long n, Entry* out)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    const auto it = g_table.find({bucket(num_taps), bucket(n)});
    if (it == g_table.end()) {
        return false;
    }
    *out = it->second;
    return true;
}

}  // namespace

// Built-in rule before tuning: the tensor-core form once the filter is long enough for FP32
// FMA throughput to bound the plain kernel (measured on GB300: plain is HBM-bound and faster up
// to about 130 taps, the tensor-core form from about 250) and the input fills the GPU; the
// plain kernel otherwise.
int tuned_fir_impl(int num_taps, long long n)
{
    Entry e;
    if (lookup(num_taps, n, &e)) {
        return e.impl;
    }
    constexpr int kTcMinTaps = 160;
    constexpr long long kTcMinSamples = 1LL << 16;
    return num_taps >= kTcMinTaps && n >= kTcMinSamples && fir_tc_supported(num_taps)
               ? RFX_FIR_TC
               : RFX_FIR_PLAIN;
}

TcConfig tuned_fir_tc_config(int num_taps, long long n)
{
    Entry e;
    if (lookup(num_taps, n, &e) && e.impl == RFX_FIR_TC) {
        return e.config;
    }
    return TcConfig{96, 6};
}

}  // namespace rfx

extern "C" int rfx_autotune_fir(int impl, int num_taps, int64_t num_samples, double* best_ms)
{
    using namespace rfx;
    if (num_taps < 1 || num_taps > kMaxTaps || num_samples < 1 || num_samples > INT32_MAX) {
        return RFX_ERR_INVALID;
    }
    void* x = nullptr;
    void* y = nullptr;
    float* h = nullptr;
    const size_t bytes = static_cast<size_t>(num_samples) * 8;
    if (cudaMalloc(&x, bytes) != cudaSuccess || cudaMalloc(&y, bytes) != cudaSuccess ||
        cudaMalloc(&h, sizeof(float) * num_taps) != cudaSuccess) {
        cudaFree(x);
        cudaFree(y);
        cudaFree(h);
        return RFX_ERR_CUDA;
    }
    cudaMemset(x, 0, bytes);
    cudaMemset(h, 0, sizeof(float) * num_taps);
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
    }
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    Entry best{RFX_FIR_PLAIN, TcConfig{96, 6}, 1e30};
    for (const Candidate& c : candidates) {
        auto run = [&]() {
            return c.impl == RFX_FIR_TC
                       ? fir_tc_launch(x, h, y, num_samples, num_taps, c.config, nullptr)
                       : fir_plain_launch(x, h, y, num_samples, num_taps, nullptr);
        };
        if (run() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
            cudaGetLastError();
            continue;  // a candidate this device cannot run is skipped
        }
        float best_c = 1e30f;
        for (int rep = 0; rep < 5; ++rep) {
            cudaEventRecord(a, nullptr);
            run();
            cudaEventRecord(b, nullptr);
            cudaEventSynchronize(b);
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            best_c = ms < best_c ? ms : best_c;
        }
        if (best_c < best.ms) {
            best = Entry{c.impl, c.config, best_c};
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(x);
    cudaFree(y);
    cudaFree(h);
    if (best.ms >= 1e29) {
        return RFX_ERR_CUDA;
    }
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        g_table[{bucket(num_taps), bucket(num_samples)}] = best;
    }
    if (best_ms != nullptr) {
        *best_ms = best.ms;
    }
    return RFX_OK;
}

namespace {

std::string device_key()
{
    int dev = 0;
    cudaDeviceProp prop{};
    int driver = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
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

}  // namespace

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
    for (const auto& kv : g_table) {
        std::fprintf(f, "%s %d %d %d %d %d %.6f\n", key.c_str(), kv.first.first, kv.first.second,
                     kv.second.impl, kv.second.config.tile_blocks, kv.second.config.stages,
                     kv.second.ms);
    }
    std::fclose(f);
    return RFX_OK;
}

extern "C" int rfx_autotune_load(const char* path)
{
    using namespace rfx;
    if (path == nullptr) {
        return RFX_ERR_INVALID;
    }
    FILE* f = std::fopen(path, "r");
    if (f == nullptr) {
        return RFX_ERR_INVALID;
    }
    const std::string key = device_key();
    char dev[256];
    int tb, lb, impl, blocks, stages;
    double ms;
    std::lock_guard<std::mutex> lock(g_mutex);
    while (std::fscanf(f, "%255s %d %d %d %d %d %lf", dev, &tb, &lb, &impl, &blocks, &stages,
                       &ms) == 7) {
        if (key == dev && (impl == RFX_FIR_PLAIN || impl == RFX_FIR_TC)) {
            g_table[{tb, lb}] = Entry{impl, TcConfig{blocks, stages}, ms};
        }
    }
    std::fclose(f);
    return RFX_OK;
}
