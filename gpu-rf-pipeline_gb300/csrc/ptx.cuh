// Inline-PTX helpers for sm_103a: mbarriers with bounded waits, bulk (TMA) copies, packed
// f32x2 arithmetic, proxy fences. Every wait here gives up after kWaitLimitNs and reports it
// through a fault word instead of spinning forever.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rfx {

// Longest a device-side wait may take before the kernel gives up (nanoseconds of %globaltimer).
// Normal waits in these kernels last microseconds; a second means something is broken.
constexpr unsigned long long kWaitLimitNs = 1000000000ull;

// Fault codes a kernel ORs into its fault word (rfx_device_fault reports them).
enum FaultCode : unsigned int {
    kFaultTileLoad = 1u << 0,     // bulk copy of an input tile never completed
    kFaultStageFull = 1u << 1,    // MMA issuer waited too long for a staged operand
    kFaultStageEmpty = 1u << 2,   // producer waited too long for a free stage
    kFaultAccumFull = 1u << 3,    // epilogue waited too long for an accumulator
    kFaultAccumEmpty = 1u << 4,   // MMA issuer waited too long for a drained accumulator
    kFaultScale = 1u << 5,        // epilogue waited too long for a tile scale
    kFaultTeardown = 1u << 6,     // final MMA commit never arrived
    kFaultPeer = 1u << 7,         // a CTA of the cluster never handed over its part
};

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---- mbarrier --------------------------------------------------------------------------

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes mbarrier initialization visible to the async proxy (bulk copies, tensor cores).
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for phase `parity` of the barrier to complete. Returns false (and ORs `code` into
// *fault) if it has not after kWaitLimitNs, or at once if *abort is already set; a give-up also
// sets *abort so the other roles of the block stop waiting too.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity,
                                                  unsigned int* fault, unsigned int code,
                                                  volatile int* abort)
{
    if (mbar_try_wait(bar, parity)) {
        return true;
    }
    const unsigned long long start = globaltimer_ns();
    while (true) {
        if (mbar_try_wait(bar, parity)) {
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

// ---- thread-block clusters -------------------------------------------------------------

__device__ __forceinline__ uint32_t cluster_ctarank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// The shared::cluster address of this CTA's shared address `addr` in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t cluster_map(uint32_t addr, uint32_t rank)
{
    uint32_t d;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(addr), "r"(rank));
    return d;
}

__device__ __forceinline__ void st_cluster_u32(uint32_t addr, uint32_t v)
{
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

// Arrives on a barrier in another CTA of the cluster (shared::cluster address), releasing this
// thread's earlier writes at cluster scope.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar)
{
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(bar)
                 : "memory");
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

// mbar_wait_bounded for a barrier that threads of other CTAs arrive on (acquire at cluster
// scope, so their writes before the arrival are visible).
__device__ __forceinline__ bool mbar_wait_cluster_bounded(uint32_t bar, uint32_t parity,
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

// Every thread of every CTA of the cluster arrives, then waits for all (the hardware barrier;
// reached once after set-up and once before exit by all threads, never skipped).
__device__ __forceinline__ void cluster_sync_all()
{
    asm volatile("barrier.cluster.arrive.release;\n\t"
                 "barrier.cluster.wait.acquire;" ::: "memory");
}

// ---- bulk copies (TMA engine, no tensor map) -------------------------------------------

// global -> shared, completion counted on `bar` in bytes. dst/src 16-byte aligned, bytes % 16 == 0.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}

// shared -> global, tracked by the issuing thread's bulk-group.
__device__ __forceinline__ void bulk_s2g(void* dst, uint32_t src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst),
                 "r"(src), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;"); }

// Waits until every committed shared->global copy of this thread has finished READING shared
// memory (the hardware completes it; no unbounded software spin).
__device__ __forceinline__ void bulk_wait_read_all()
{
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// Orders this thread's generic-proxy shared-memory accesses before later async-proxy accesses
// (bulk copies, tensor-core operand reads).
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---- packed f32x2 arithmetic -----------------------------------------------------------

// A pair of float32 values in one 64-bit register: low word first (I), high word second (Q).
using f32x2 = unsigned long long;

__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c)
{
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

__device__ __forceinline__ f32x2 pack2(float lo, float hi)
{
    f32x2 d;
    asm("mov.b64 %0, {%1, %2};" : "=l"(d) : "f"(lo), "f"(hi));
    return d;
}

__device__ __forceinline__ float2 unpack2(f32x2 v)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(v));
    return r;
}

__device__ __forceinline__ f32x2 lds64(uint32_t addr)
{
    f32x2 v;
    asm volatile("ld.shared.b64 %0, [%1];" : "=l"(v) : "r"(addr));
    return v;
}

__device__ __forceinline__ void sts64(uint32_t addr, f32x2 v)
{
    asm volatile("st.shared.b64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

// ---- per-thread asynchronous copies (global -> shared) ----------------------------------

// kBytes (4, 8 or 16) bytes from src to shared address dst; src_bytes = 0 reads nothing and
// writes zeros.
template <int kBytes>
__device__ __forceinline__ void cp_async(uint32_t dst, const void* src, uint32_t src_bytes)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(dst), "l"(src),
                 "n"(kBytes), "r"(src_bytes)
                 : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

// Waits until at most kPending of this thread's committed copy groups are still in flight.
template <int kPending>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;" ::"n"(kPending) : "memory");
}

}  // namespace rfx
