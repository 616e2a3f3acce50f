// Bulk asynchronous copies (TMA, untiled cp.async.bulk) into shared memory,
// completed on an mbarrier, with bounded waits.
//
// Rules the callers keep: source and destination addresses 16-byte aligned,
// sizes multiples of 16 bytes; the barrier is initialised (count 1: the
// issuing thread's arrive.expect_tx) and the init fenced before any wait;
// a buffer is refilled only after every thread's reads of it are done
// (a CTA barrier), followed by fence_proxy_async_smem() in the issuing
// thread, which orders those generic-proxy reads before the async-proxy
// writes.
#pragma once

#include <cstdint>

namespace bem {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes the barrier inits visible to the async proxy and the cluster.
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Arrive (count 1) and add `bytes` to the transaction count of the phase.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// True once the phase of the given parity has completed (may suspend the
// thread for a bounded, hardware-chosen time before returning false).
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits at most `limit` SM clock cycles (plus one try_wait) for the phase;
// false on timeout, or at once when *abort is set by another thread.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, long long limit,
                                                  volatile int *abort) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (*abort || clock64() - t0 > limit) return false;
    }
    return true;
}

// global -> this CTA's shared memory, `bytes` (multiple of 16) completing on bar.
__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Plain arrive (count 1, release semantics) on an mbarrier.
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Distributed shared memory: the shared::cluster address of p in CTA rank.
__device__ __forceinline__ uint32_t cluster_addr(const void *p, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    return r;
}
// 8 bytes into another CTA's shared memory, completing on its mbarrier.
__device__ __forceinline__ void st_async_f2(uint32_t addr, float2 v, uint32_t bar) {
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v2.f32 [%0], {%1, %2}, [%3];" ::"r"(addr),
                 "f"(v.x), "f"(v.y), "r"(bar)
                 : "memory");
}
// Bounded wait with cluster-scope acquire (the bytes came from other CTAs).
__device__ __forceinline__ bool mbar_wait_cluster_bounded(uint64_t *bar, uint32_t parity, long long limit,
                                                          volatile int *abort) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        if (*abort || clock64() - t0 > limit) return false;
    }
}

}  // namespace bem
