// async.cuh -- mbarrier, bulk-copy and timer helpers (inline PTX, sm_90+ forms
// that sm_103a keeps).  Every wait is bounded.
#pragma once

#include <stdint.h>

namespace sphfem {

constexpr unsigned long long kWaitNs = 1000000000ull;   // 1 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// One-arrival mbarrier, initialised and made visible to the async proxy.
__device__ __forceinline__ void mbar_init(uint32_t mbar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(1) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Bounded wait for the phase `parity` of the mbarrier to complete (1 s).
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity) {
    const unsigned long long t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 26); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if ((it & 63) == 63 && global_ns() - t0 > kWaitNs) return false;
    }
    return false;
}

// The arrival of the issuing thread, announcing `bytes` of bulk copies.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// Contiguous global -> shared copy by the bulk-copy engine; completes bytes on
// the mbarrier.  Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(uint32_t dst_smem, const void *src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     dst_smem),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}

// Hint to the bulk-copy engine: bring [p, p + bytes) into L2.  No completion,
// nothing to wait for.  Skipped unless p is non-null and 16-byte aligned; bytes
// rounded down to a multiple of 16.
__device__ __forceinline__ void prefetch_l2_bulk(const void *p, uint32_t bytes) {
    bytes &= ~15u;
    if (!p || bytes == 0 || ((uintptr_t)p & 15u)) return;
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

}  // namespace sphfem
