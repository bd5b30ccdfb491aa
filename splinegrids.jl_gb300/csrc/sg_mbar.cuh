// sg_mbar.cuh -- shared-memory barriers (mbarrier) and bulk copies (cp.async.bulk, the
// Tensor Memory Accelerator's untiled form) for the streaming kernels.
//
// Every wait is bounded in time and also gives up when the CTA's abort flag is set,
// so a copy that never completes ends in an error status instead of a hang.
#pragma once

#include "sg_common.cuh"

namespace sg {

constexpr long long kMbarWaitCycles = 2000000000ll;  // ~1 s at the maximum SM clock

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

// makes the initialized barriers visible to the async proxy (bulk copies)
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// adds `bytes` of expected transaction count to the current phase without arriving
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Test for the completion of the phase with the given parity.  The suspend-time hint
// lets the hardware park the thread until the phase completes (or ~1 ms passes)
// instead of returning at once: waiting warps then take no issue slots from the warps
// on the same scheduler that do the work.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(1000000u)
        : "memory");
    return ok != 0;
}

// Wait for the completion of the barrier's phase with the given parity.  Returns
// false, without waiting further, after kMbarWaitCycles SM clock cycles or once
// *abort (when given) is nonzero.  The SM cycle counter is cheap to read, so polls
// follow each other closely.
__device__ __forceinline__ bool mbar_wait_for(uint64_t *bar, unsigned parity, volatile int *abort,
                                              long long cycles) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((abort && *abort) || clock64() - t0 > cycles) return false;
    }
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity, volatile int *abort) {
    return mbar_wait_for(bar, parity, abort, kMbarWaitCycles);
}

// global -> shared bulk copy completing `bytes` of transaction count on `bar`
// (addresses and size 16-byte aligned)
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// orders this thread's earlier generic-proxy accesses of shared memory before its
// later async-proxy (bulk copy) accesses
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// orders global-memory writes observed through the generic proxy (other CTAs' stores,
// acquired on a counter) before later bulk-copy reads of this thread
__device__ __forceinline__ void fence_proxy_async_global() {
    asm volatile("fence.proxy.async.global;\n" ::: "memory");
}

}  // namespace sg
