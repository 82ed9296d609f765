#pragma once

// Test harness: a small runtime with the member functions that code generated by the project's
// SigFlow compiler calls (its CUDA backend, compiler/src/backend_cuda.cpp:108-175, :209-290,
// emits calls on a `sigflow::Runtime rt`). It exists so that a program shaped like that
// generated code compiles against this library's device_ops.hpp and runs; the project's own
// runtime (src/pipeline_runtime.*) does the same jobs with its own reporting.
//
// Buffers: numbered slots, each sized to the largest `need` it was given, one cudaMalloc each.
// Paths are relative to the working directory. `run` runs upload, compute and download once,
// then synchronizes; `report` prints the kernel counts as JSON.

#include "check.hpp"
#include "types.hpp"

#include <cufft.h>

#include <cstdio>
#include <fstream>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace sigflow {

inline std::size_t padded_to_frames(std::size_t n, int frame)
{
    return (n + static_cast<std::size_t>(frame) - 1) / frame * frame;
}

class Runtime {
public:
    Runtime(const char* program, const char* kernels, bool fused, bool reuse, int, char**)
        : program_(program), kernels_(kernels), fused_(fused), reuse_(reuse)
    {
    }

    ~Runtime()
    {
        for (auto& kv : plans_) {
            cufftDestroy(kv.second);
        }
        for (void* p : owned_) {
            cudaFree(p);
        }
    }

    Runtime(const Runtime&) = delete;
    Runtime& operator=(const Runtime&) = delete;

    std::vector<cf32> read_capture(const std::string& path) { return load<cf32>(path); }

    void need(int slot, std::size_t bytes)
    {
        std::size_t& have = sizes_[slot];
        have = bytes > have ? bytes : have;
    }

    void allocate_slots()
    {
        for (const auto& kv : sizes_) {
            void* p = nullptr;
            CUDA_CHECK(cudaMalloc(&p, kv.second > 0 ? kv.second : 16));
            owned_.push_back(p);
            slots_[kv.first] = p;
        }
    }

    template <class T>
    T* slot(int index)
    {
        return static_cast<T*>(slots_.at(index));
    }

    const float* taps(const std::string& path, int& count)
    {
        const std::vector<float> h = load<float>(path);
        if (h.empty()) {
            throw std::runtime_error(path + ": no taps");
        }
        void* p = nullptr;
        CUDA_CHECK(cudaMalloc(&p, h.size() * sizeof(float)));
        owned_.push_back(p);
        CUDA_CHECK(cudaMemcpy(p, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
        count = static_cast<int>(h.size());
        return static_cast<const float*>(p);
    }

    cufftHandle fft_plan(int points, std::size_t frames)
    {
        cufftHandle plan{};
        CUFFT_CHECK(cufftPlan1d(&plan, points, CUFFT_C2C, static_cast<int>(frames)));
        plans_[static_cast<int>(plans_.size())] = plan;
        return plan;
    }

    void run(const std::function<void()>& upload, const std::function<void()>& compute,
             const std::function<void()>& download)
    {
        upload();
        compute();
        CUDA_CHECK(cudaGetLastError());
        download();
        CUDA_CHECK(cudaDeviceSynchronize());
    }

    void count(const char* kernel) { ++counts_[kernel]; }

    void write_cf32(const std::string& path, const std::vector<cf32>& v) { save(path, v); }
    void write_f32(const std::string& path, const std::vector<float>& v) { save(path, v); }

    void report() const
    {
        std::printf("{\"program\": \"%s\", \"kernels\": \"%s\", \"fused\": %s, \"reuse\": %s, "
                    "\"launches\": {",
                    program_.c_str(), kernels_.c_str(), fused_ ? "true" : "false",
                    reuse_ ? "true" : "false");
        bool first = true;
        for (const auto& kv : counts_) {
            std::printf("%s\"%s\": %d", first ? "" : ", ", kv.first.c_str(), kv.second);
            first = false;
        }
        std::printf("}}\n");
    }

private:
    template <class T>
    static std::vector<T> load(const std::string& path)
    {
        std::ifstream f(path, std::ios::binary | std::ios::ate);
        if (!f) {
            throw std::runtime_error(path + ": cannot open");
        }
        const std::streamsize bytes = f.tellg();
        f.seekg(0);
        std::vector<T> v(static_cast<std::size_t>(bytes) / sizeof(T));
        f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
        return v;
    }

    template <class T>
    static void save(const std::string& path, const std::vector<T>& v)
    {
        std::ofstream f(path, std::ios::binary);
        if (!f) {
            throw std::runtime_error(path + ": cannot write");
        }
        f.write(reinterpret_cast<const char*>(v.data()),
                static_cast<std::streamsize>(v.size() * sizeof(T)));
    }

    std::string program_, kernels_;
    bool fused_, reuse_;
    std::map<int, std::size_t> sizes_;
    std::map<int, void*> slots_;
    std::vector<void*> owned_;
    std::map<int, cufftHandle> plans_;
    std::map<std::string, int> counts_;
};

}  // namespace sigflow
