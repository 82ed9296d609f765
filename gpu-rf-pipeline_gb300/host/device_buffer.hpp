#pragma once

// Owning device buffer with blocking upload / download (src/device_buffer.hpp:11-76 semantics).

#include "check.hpp"

#include <cstddef>
#include <cstdio>

template <class T>
class DeviceBuffer {
public:
    explicit DeviceBuffer(std::size_t count) : count_(count)
    {
        if (count_ > 0) {
            CUDA_CHECK(cudaMalloc(&ptr_, count_ * sizeof(T)));
        }
    }
    ~DeviceBuffer()
    {
        if (ptr_ != nullptr) {
            const cudaError_t err = cudaFree(ptr_);
            if (err != cudaSuccess) {
                std::fprintf(stderr, "warning: cudaFree failed: %s\n", cudaGetErrorString(err));
            }
        }
    }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;

    T* get() const { return ptr_; }
    std::size_t size() const { return count_; }

    void upload(const T* host, std::size_t count)
    {
        if (count > 0) {
            CUDA_CHECK(cudaMemcpy(ptr_, host, count * sizeof(T), cudaMemcpyHostToDevice));
        }
    }
    void download(T* host, std::size_t count) const
    {
        if (count > 0) {
            CUDA_CHECK(cudaMemcpy(host, ptr_, count * sizeof(T), cudaMemcpyDeviceToHost));
        }
    }
    void zero()
    {
        if (count_ > 0) {
            CUDA_CHECK(cudaMemset(ptr_, 0, count_ * sizeof(T)));
        }
    }

private:
    T* ptr_ = nullptr;
    std::size_t count_ = 0;
};
