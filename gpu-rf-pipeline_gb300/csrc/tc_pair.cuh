// CTA-pair (cluster of two) helpers for sm_103a: 2-SM tcgen05 MMAs, tensor-memory allocation
// for the pair, multicast commits, and mbarrier operations across the pair.
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

__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Every thread of both CTAs; release/acquire at cluster scope.
__device__ __forceinline__ void cluster_sync()
{
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n\t"
        "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Shared-memory address of the same variable in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t map_to(uint32_t addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

// Arrive (release, cluster scope) on an mbarrier given by its cluster address.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t cluster_addr)
{
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(cluster_addr)
                 : "memory");
}

__device__ __forceinline__ void st_cluster_u32(uint32_t cluster_addr, uint32_t v)
{
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(cluster_addr), "r"(v) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait_cluster(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// mbar_wait_bounded with acquire at cluster scope (the barrier's arrivals may come from the
// other CTA of the pair).
__device__ __forceinline__ bool mbar_wait_cluster(uint32_t bar, uint32_t parity,
                                                  unsigned int* fault, unsigned int code,
                                                  volatile int* abort)
{
    if (mbar_try_wait_cluster(bar, parity)) {
        return true;
    }
    const unsigned long long start = globaltimer_ns();
    while (true) {
        if (mbar_try_wait_cluster(bar, parity)) {
            return true;
        }
        if (abort != nullptr && *abort) {
            return false;
        }
        if (globaltimer_ns() - start > kWaitLimitNs) {
            atomicOr(fault, code);
            if (abort != nullptr) {
                *abort = 1;
            }
            return false;
        }
    }
}

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
