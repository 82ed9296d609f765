#pragma once

// Error checking that throws std::runtime_error with the failing call, the library's message
// and the source location, as the project's CUDA_CHECK / CUFFT_CHECK do (src/check.hpp:42-66).
// RFX_CHECK does the same for a status returned by the C ABI (include/rfx.h).

#include "rfx.h"

#include <cuda_runtime.h>
#include <cufft.h>

#include <stdexcept>
#include <string>

[[noreturn]] inline void throw_call_error(const char* library, const std::string& text, int code,
                                          const char* call, const char* file, int line)
{
    throw std::runtime_error(std::string(library) + " error: " + text + " (code " +
                             std::to_string(code) + ")\n  in: " + call + "\n  at: " + file + ":" +
                             std::to_string(line));
}

#define CUDA_CHECK(call)                                                                        \
    do {                                                                                        \
        const cudaError_t cuda_check_err_ = (call);                                             \
        if (cuda_check_err_ != cudaSuccess) {                                                   \
            throw_call_error("CUDA", cudaGetErrorString(cuda_check_err_),                       \
                             static_cast<int>(cuda_check_err_), #call, __FILE__, __LINE__);     \
        }                                                                                       \
    } while (0)

#define CUFFT_CHECK(call)                                                                       \
    do {                                                                                        \
        const cufftResult cufft_check_err_ = (call);                                            \
        if (cufft_check_err_ != CUFFT_SUCCESS) {                                                \
            throw_call_error("cuFFT", "cufftResult", static_cast<int>(cufft_check_err_), #call, \
                             __FILE__, __LINE__);                                               \
        }                                                                                       \
    } while (0)

#define RFX_CHECK(call)                                                                         \
    do {                                                                                        \
        const int rfx_check_status_ = (call);                                                   \
        if (rfx_check_status_ != RFX_OK) {                                                      \
            throw_call_error("rfx", rfx_last_error(), rfx_check_status_, #call, __FILE__,       \
                             __LINE__);                                                         \
        }                                                                                       \
    } while (0)
