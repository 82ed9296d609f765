// Sample formats of the FIR kernels' input and their decoding where the samples are staged.
//
// 0 = cf32 (interleaved float32 I, Q); 1 = ci16 and 2 = ci8 (interleaved signed integer I, Q as
// stored by SDR receivers). Integer components decode as the project's SigMF reader converts
// them (src/io.cpp:110-148): v / 32768 and v / 128, both exact in float32, so a kernel that
// decodes in its load stage gives the bits of a run over the host-converted samples.
#pragma once

#include "tc_common.cuh"

#include <cstdint>

namespace rfx {
namespace tc {

__host__ __device__ constexpr int component_bytes(int fmt) { return fmt == 0 ? 4 : fmt == 1 ? 2 : 1; }

__device__ __forceinline__ float4 decode_ci16x2(uint2 w)
{
    constexpr float k = 1.0f / 32768.0f;
    return make_float4(static_cast<float>(static_cast<int>(w.x << 16) >> 16) * k,
                       static_cast<float>(static_cast<int>(w.x) >> 16) * k,
                       static_cast<float>(static_cast<int>(w.y << 16) >> 16) * k,
                       static_cast<float>(static_cast<int>(w.y) >> 16) * k);
}

__device__ __forceinline__ float4 decode_ci8x2(uint32_t w)
{
    constexpr float k = 1.0f / 128.0f;
    return make_float4(static_cast<float>(static_cast<int>(w << 24) >> 24) * k,
                       static_cast<float>(static_cast<int>(w << 16) >> 24) * k,
                       static_cast<float>(static_cast<int>(w << 8) >> 24) * k,
                       static_cast<float>(static_cast<int>(w) >> 24) * k);
}

// Samples s, s + 1 (s even) from shared memory holding components in format fmt at `addr`
// (the first of the pair): re0, im0, re1, im1.
__device__ __forceinline__ float4 lds_pair(uint32_t addr, int fmt)
{
    if (fmt == 0) {
        return lds128(addr);
    }
    if (fmt == 1) {
        uint2 w;
        asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(w.x), "=r"(w.y) : "r"(addr) : "memory");
        return decode_ci16x2(w);
    }
    uint32_t w;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(w) : "r"(addr) : "memory");
    return decode_ci8x2(w);
}

// Samples s, s + 1 of x (s even, s + 1 < n), and sample s alone, from global memory.
__device__ __forceinline__ float4 ldg_pair(const void* x, int fmt, long long s)
{
    if (fmt == 0) {
        return __ldg(reinterpret_cast<const float4*>(static_cast<const float2*>(x) + s));
    }
    if (fmt == 1) {
        return decode_ci16x2(__ldg(reinterpret_cast<const uint2*>(static_cast<const short2*>(x) + s)));
    }
    return decode_ci8x2(__ldg(reinterpret_cast<const unsigned int*>(static_cast<const char2*>(x) + s)));
}

__device__ __forceinline__ float2 ldg_one(const void* x, int fmt, long long s)
{
    if (fmt == 0) {
        return __ldg(static_cast<const float2*>(x) + s);
    }
    if (fmt == 1) {
        const short2 v = __ldg(static_cast<const short2*>(x) + s);
        return make_float2(static_cast<float>(v.x) * (1.0f / 32768.0f),
                           static_cast<float>(v.y) * (1.0f / 32768.0f));
    }
    const char2 v = __ldg(static_cast<const char2*>(x) + s);
    return make_float2(static_cast<float>(v.x) * (1.0f / 128.0f),
                       static_cast<float>(v.y) * (1.0f / 128.0f));
}

}  // namespace tc
}  // namespace rfx
