// CTA-pair (cluster of two) helpers for sm_103a: 2-SM tcgen05 MMAs, tensor-memory allocation
// for the pair and multicast commits (cluster barriers, distributed shared memory and
// cross-CTA mbarrier operations are in ptx.cuh).
//
// In a 2-SM MMA (cta_group::2, M = 256) the even CTA of the pair (rank 0) issues every MMA.
// Each CTA supplies, at the same shared-memory offsets, half of A (rank r: rows 128 r .. +127)
// and half of B (rank r: columns N/2 r .. +N/2-1); each CTA's tensor memory receives its 128
// rows of D, all N columns.
#pragma once

#include <cstdint>

#include "ptx.cuh"

namespace rfx {
namespace pair {

// One warp in EACH CTA of the pair executes these.
__device__ __forceinline__ void tmem_alloc_pair(uint32_t dst_smem, uint32_t cols)
{
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t cols)
{
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols));
}

// D (tensor memory) [+]= A B for the pair, kind::f16, FP32 accumulation.
template <uint32_t kIdesc>
__device__ __forceinline__ void mma_pair(uint32_t d_tmem, unsigned long long a, unsigned long long b,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
        : "memory");
}

// Arrives once on the mbarrier at this shared-memory offset in both CTAs of the pair when every
// MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit_pair(uint32_t bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 "
        "[%0], %1;" ::"r"(bar),
        "h"(static_cast<unsigned short>(3))
        : "memory");
}

}  // namespace pair
}  // namespace rfx
