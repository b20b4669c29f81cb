// Bulk (TMA) staging of read-only per-step tables into shared memory:
// cp.async.bulk global -> shared with an mbarrier counting the bytes.
//
// Rules kept here: source and destination 16-byte aligned, sizes multiples of
// 16 bytes (the tables are padded to that), at most 2^20 - 1 bytes per
// mbarrier phase. The wait is bounded: after kStageSpin polls the caller gets
// `false` and must not read the destination.
#pragma once
#include <cstdint>

namespace nqes {

constexpr long long kStageSpin = 1LL << 24;

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

// One bulk copy of `bytes` (multiple of 16) from global to shared memory.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, uint64_t *mbar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(mbar))
        : "memory");
}

// Bounded wait for phase `parity` of the mbarrier: at most `polls` polls;
// false when it ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, unsigned parity, long long polls = kStageSpin) {
    for (long long it = 0; it < polls; it++) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(mbar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

}  // namespace nqes
