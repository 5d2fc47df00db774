// tt_tma.cuh — bulk (TMA) global->shared copies completed on an mbarrier.
//
// Every wait is bounded: after kSpinLimit polls the waiting thread records
// TT_DEV_ERR_TIMEOUT in the kernel's error word and carries on, so a lost
// completion can never hang the GPU; the host turns the word into
// TT_ERR_TIMEOUT.
#pragma once
#include "tt_common.cuh"

namespace tt {

constexpr u32 TT_DEV_ERR_TIMEOUT = 1u;
constexpr u32 kSpinLimit = 1u << 24;

__device__ __forceinline__ u32 smem_addr(const void* p) {
    return static_cast<u32>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(u64* bar, u32 count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(u64* bar, u32 bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// Bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned) from
// global to shared memory, completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, u32 bytes, u64* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

// Wait for phase `parity` of `bar` to complete; bounded. On a timeout the
// error word gets TT_DEV_ERR_TIMEOUT and, if given, the CTA-local flag
// `local` (shared memory) becomes 1, so the CTA can stop without polling
// global memory.
__device__ __forceinline__ void mbar_wait(u64* bar, u32 parity, u32* err, volatile u32* local = nullptr) {
    const u32 a = smem_addr(bar);
    for (u32 i = 0; i < kSpinLimit; ++i) {
        u32 done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return;
    }
    if (err) atomicOr(err, TT_DEV_ERR_TIMEOUT);
    if (local) *local = 1u;
}

}  // namespace tt
