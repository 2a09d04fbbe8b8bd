// rt_tma.cuh — bulk asynchronous copies (TMA, cp.async.bulk) and mbarriers for sm_103a.
//
// Used by the STAGED fold: one thread issues 1-D bulk copies global -> shared that complete on an
// mbarrier's transaction count, so a block keeps many kilobytes in flight without holding them in
// registers.  No multicast, no cluster launch: the shared::cluster forms address this CTA's own
// shared memory.  Every wait is bounded by the runtime's timeout.
#pragma once
#include "rt_core.cuh"

namespace gpumpi {

// Dynamic shared memory of the rank kernel (size chosen per launch by the host; c_rt.dyn_smem).
extern __shared__ __align__(128) unsigned char g_dyn_smem[];

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(unsigned long long* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders this thread's view of global memory (generic proxy, e.g. data published by other ranks before
// an acquire) before its later bulk copies (async proxy) read it
__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// 1-D bulk copy of `bytes` (multiple of 16; both addresses 16-byte aligned) into this CTA's shared memory.
__device__ __forceinline__ void tma_load_1d(void* smem_dst, const void* gsrc, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(smem_dst)),
        "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of parity `parity` to complete; false if it did not within the runtime timeout.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long end = now_ns() + (unsigned long long)c_rt.timeout_ns;
    for (unsigned i = 1;; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 63u) == 0 && now_ns() > end) return false;
    }
}

}  // namespace gpumpi
