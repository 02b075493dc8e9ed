// Bulk asynchronous copies global -> shared memory (cp.async.bulk, the TMA
// unit's untiled form) completed on a shared-memory mbarrier, and a bounded
// wait on that barrier.  Rules of the untiled copy: source and destination
// 16-byte aligned, size a multiple of 16 bytes.
#pragma once

#include <stdint.h>

namespace pyl {

__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}

// Makes initialised barriers visible to the async proxy (the copy engine).
__device__ __forceinline__ void mbar_init_fence() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy ones (a buffer read by threads, then refilled by a copy).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One arrival that also announces `bytes` of transactions to come.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, unsigned bytes,
                                              uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_test_parity(uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n"
        "  .reg .pred p;\n"
        "  mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "  selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of the given parity to complete; gives up (false)
// after about one second so that a lost copy cannot hang the GPU.
constexpr uint64_t kWaitLimitNs = 1000000000ull;
__device__ __forceinline__ bool mbar_wait_parity(uint64_t *bar, unsigned parity) {
    if (mbar_test_parity(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    while (!mbar_test_parity(bar, parity))
        if (global_ns() - t0 > kWaitLimitNs) return false;
    return true;
}

// Device status word bits (pyl_ctx::d_status), read back by the host at its
// next synchronisation point.
constexpr unsigned kStatusWaitTimeout = 1u;
// The exact tile sort found particles that its counting pass had not
// counted where they landed: the positions changed between its passes (a
// caller still writing them on another stream).  The overflowing particles
// are dropped, the deposit is skipped, and the call reports an error.
constexpr unsigned kStatusInputChanged = 2u;
// A kernel met a bound its launch should have ruled out (a sort's chunk
// table): it wrote nothing, the deposit is skipped and the call fails.
constexpr unsigned kStatusInternal = 4u;

}  // namespace pyl
