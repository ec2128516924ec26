/*
 * bulk_copy.cuh -- one-dimensional TMA bulk copies (global -> shared) with
 * mbarrier completion, for kernels that stage their next row block while they
 * work on the current one (sm_90 and later; written for sm_103a).
 *
 * Rules the callers keep: source and destination 16-byte aligned, sizes a
 * multiple of 16 bytes; one thread arms a barrier with the byte count of all
 * the copies it then issues on it; every wait is bounded in time, and a wait
 * that runs out reports it instead of spinning on.
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pdal {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

/* makes barrier initialisation visible to the async (TMA) proxy */
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

/* orders this thread's earlier generic-proxy accesses of shared memory before
 * later async-proxy writes to it (a buffer read by the block is about to be
 * refilled by a bulk copy) */
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* one arrival on the barrier plus `bytes` expected transaction bytes */
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

/* Waits for the barrier phase of parity `parity`; false when it has not
 * completed within `limit_ns` of wall time. */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > limit_ns) return false;
    }
}

/* the wall-time bound of one staging wait (a copy of a few tens of KB takes
 * microseconds; this only ends a wait that would otherwise never end) */
constexpr unsigned long long kStageWaitNs = 2000000000ull;

} // namespace pdal
