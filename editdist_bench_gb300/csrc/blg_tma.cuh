// Bulk-copy (TMA) staging helpers: mbarrier and cp.async.bulk in inline PTX.
//
// A CTA stages a contiguous byte span of global memory into its shared
// memory with one `cp.async.bulk` per span, completed on an mbarrier by
// transaction count. Rules the callers keep: global source and shared
// destination 16-byte aligned, size a multiple of 16, and every wait
// bounded (a wait that gives up reports it; the caller raises a status bit).
#pragma once
#include <stdint.h>

namespace blg {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// One thread initialises; the fences make the initialisation visible to the
// async (bulk-copy) proxy before the CTA-wide barrier that follows.
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(arrivals) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Arrive once and announce `bytes` of bulk-copy transactions for this phase
// (0 bytes: the phase completes with the arrival alone).
__device__ __forceinline__ void mbar_arrive_expect(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
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

// Bounded wait for phase `parity` of `bar`. Each try_wait suspends for a
// hardware-chosen interval, so the bound is seconds of wall time, far above
// any copy's latency. Returns false when it gave up.
constexpr uint32_t kMbarPolls = 1u << 24;

__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t polls = kMbarPolls) {
    for (uint32_t i = 0; i < polls; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Global -> shared bulk copy completed on `bar` (16-byte aligned, size % 16 == 0).
__device__ __forceinline__ void bulk_g2s(void *dst_smem, const void *src_gmem, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst_smem)),
        "l"(src_gmem), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

}  // namespace blg
