// Helpers shared by the tensor-core kernels: tcgen05 MMA issue and commit, shared-memory matrix
// descriptors, TMA tiled loads, and the scaled FP16 hi/lo split.
#pragma once

#include "ptx.cuh"

#include <cuda.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace rfx {
namespace tc {

// Shared-memory matrix descriptor, no swizzle, K-major: start address, leading-byte offset
// (stride between 8-element K groups), stride-byte offset (between 8-row groups); bits 46-48
// hold the fixed value 1 of the tcgen05 descriptor format.
__device__ __forceinline__ unsigned long long smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return static_cast<unsigned long long>((addr >> 4) & 0x3FFFu) |
           (static_cast<unsigned long long>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<unsigned long long>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16 with FP16 A and B (both K-major) and FP32 D.
constexpr uint32_t idesc_f16(int m, int n)
{
    return (1u << 4) | (static_cast<uint32_t>(n >> 3) << 17) | (static_cast<uint32_t>(m >> 4) << 24);
}

template <uint32_t kIdesc>
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, unsigned long long a,
                                        unsigned long long b, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

// The same with the accumulate flag fixed at 1 (D += A B): no predicate set-up from a register.
template <uint32_t kIdesc>
__device__ __forceinline__ void mma_f16_acc(uint32_t d_tmem, unsigned long long a,
                                            unsigned long long b)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.eq.u32 p, 1, 1;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(kIdesc)
        : "memory");
}

// One lane of a fully active warp (the same lane every time): the lane that issues a warp's
// MMAs and commits. Running the issue loop on the whole warp and electing the issuer keeps
// the loop's values (descriptors, TMEM addresses, counters) warp-uniform, so they can live in
// the uniform registers the MMA instruction reads, instead of being moved there per MMA.
__device__ __forceinline__ bool elect_one()
{
    uint32_t pred = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\telect.sync _|p, 0xffffffff;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(pred));
    return pred != 0;
}

__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}

__device__ __forceinline__ void fence_before()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t cols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols));
}

// 16 consecutive 32-bit TMEM columns of this thread's lane (32x32b shape), then wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&t)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]),
          "=r"(t[7]), "=r"(t[8]), "=r"(t[9]), "=r"(t[10]), "=r"(t[11]), "=r"(t[12]), "=r"(t[13]),
          "=r"(t[14]), "=r"(t[15])
        : "r"(taddr));
}

// 8 consecutive 32-bit TMEM columns of this thread's lane (32x32b shape); tmem_wait_ld after.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&t)[8])
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]),
                   "=r"(t[6]), "=r"(t[7])
                 : "r"(taddr));
}

// 16 lanes x 256 bits, four times along the columns: for 8-column group j (registers 4j .. 4j+3)
// thread t holds (lane t/4: columns 2 (t%4), +1) and (lane t/4 + 8: the same columns) of the 16
// lanes starting at taddr's lane.
__device__ __forceinline__ void tmem_ld_16x256b_x4(uint32_t taddr, uint32_t (&t)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.16x256b.x4.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(t[0]), "=r"(t[1]), "=r"(t[2]), "=r"(t[3]), "=r"(t[4]), "=r"(t[5]), "=r"(t[6]),
          "=r"(t[7]), "=r"(t[8]), "=r"(t[9]), "=r"(t[10]), "=r"(t[11]), "=r"(t[12]), "=r"(t[13]),
          "=r"(t[14]), "=r"(t[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld()
{
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// 2-D tiled TMA load at (x0, y0) into shared memory, completion on `bar`.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x0, int y0,
                                            uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x0), "r"(y0), "r"(bar)
        : "memory");
}

// 2^e as a float, e clamped to the normal range [-126, 127].
__device__ __forceinline__ float exp2i(int e)
{
    e = e < -126 ? -126 : (e > 127 ? 127 : e);
    return __int_as_float((e + 127) << 23);
}

// 2^e as a float for e in [-149, 127] (subnormal below -126), exact.
__device__ __forceinline__ float exp2_exact(int e)
{
    return e >= -126 ? __int_as_float((e + 127) << 23) : __int_as_float(1 << (e + 149));
}

// Exponent that brings a magnitude with these float bits into [2^14, 2^15): 141 - biased
// exponent; 0 for zero.
__device__ __forceinline__ int scale_exponent(uint32_t abs_bits)
{
    return abs_bits == 0 ? 0 : 141 - static_cast<int>((abs_bits >> 23) & 0xFFu);
}

// FP16 hi/lo split of two values already scaled into range: hi = fp16(v), lo = fp16(v - hi).
__device__ __forceinline__ void split2(float a, float b, uint32_t& hi, uint32_t& lo)
{
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t*>(&h);
    lo = *reinterpret_cast<const uint32_t*>(&l);
}

__device__ __forceinline__ void sts32(uint32_t addr, uint32_t v)
{
    asm volatile("st.shared.b32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

__device__ __forceinline__ float4 lds128(uint32_t addr)
{
    float4 v;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
                 : "r"(addr)
                 : "memory");
    return v;
}

__device__ __forceinline__ uint32_t absbits(float v) { return __float_as_uint(v) & 0x7FFFFFFFu; }

__device__ __forceinline__ uint32_t absmax4(float4 v)
{
    return max(max(absbits(v.x), absbits(v.y)), max(absbits(v.z), absbits(v.w)));
}

}  // namespace tc
}  // namespace rfx
