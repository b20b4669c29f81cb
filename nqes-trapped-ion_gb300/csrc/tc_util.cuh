// Fifth-generation tensor cores (tcgen05) on sm_103a: tensor-memory
// allocation, shared-memory matrix descriptors, the BF16 MMA with FP32
// accumulation, its completion on an mbarrier and tensor-memory loads.
//
// Operand layout used throughout: K-major without swizzling. A matrix of R
// rows and KP columns (KP a multiple of 16 bf16) is stored as 8 x 8 core
// matrices of 128 contiguous bytes (8 rows x 16 bytes); core matrices
// adjacent along K are 128 bytes apart (leading byte offset), 8-row groups
// are KP * 16 bytes apart (stride byte offset):
//     byte(r, c) = (r / 8) * KP * 16 + (c / 8) * 128 + (r % 8) * 16 + (c % 8) * 2.
// One MMA consumes K = 16 (two core matrices along K); the next K step starts
// 256 bytes further.
//
// Accumulator D (M = 128 rows) occupies tensor-memory lanes 0..127 (row m in
// lane m) and N consecutive 32-bit columns; warp w of the CTA may read lanes
// 32 (w % 4) .. 32 (w % 4) + 31.
#pragma once
#include <cstdint>

#include "tma_stage.cuh"

namespace nqes {

__host__ __device__ constexpr int round16(int x) { return (x + 15) & ~15; }

// byte offset of element (r, c) in a K-major, unswizzled operand of KP columns
__host__ __device__ inline unsigned kmajor_off(int r, int c, int KP) {
    return unsigned((r >> 3) * KP * 16 + (c >> 3) * 128 + (r & 7) * 16 + (c & 7) * 2);
}

// Shared-memory matrix descriptor: start address, leading byte offset (along
// K), stride byte offset (along M/N), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(const void *base, unsigned lbo, unsigned sbo) {
    const uint64_t a = smem_u32(base);
    uint64_t d = 0;
    d |= (a >> 4) & 0x3FFFULL;
    d |= uint64_t((lbo >> 4) & 0x3FFF) << 16;
    d |= uint64_t((sbo >> 4) & 0x3FFF) << 32;
    d |= 1ULL << 46;  // version
    return d;         // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4)                       // D format: F32
           | (1u << 7)                     // A format: BF16
           | (1u << 10)                    // B format: BF16
           | (uint32_t(N >> 3) << 17)      // N / 8
           | (uint32_t(M >> 4) << 24);     // M / 16
}

// Tensor-memory allocation by one whole warp; the address lands in *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, unsigned ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, unsigned ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D (+)= A B^T for one K step of 16, issued by a single thread.
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate ? 1u : 0u)
        : "memory");
}

// The mbarrier receives one arrival when every MMA issued so far by this
// thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t *mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the tensor cores
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive 32-bit columns of this thread's lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

// x = hi + mid + lo exactly, each a BF16 (truncation keeps 8 significant bits
// per term: 24 in all, the whole FP32 significand). Returned as BF16 bits.
__device__ __forceinline__ void bf16_split3_trunc(float x, uint32_t &hi, uint32_t &mid, uint32_t &lo) {
    const uint32_t b = __float_as_uint(x) & 0xFFFF0000u;
    const float r1 = x - __uint_as_float(b);
    const uint32_t m = __float_as_uint(r1) & 0xFFFF0000u;
    const float r2 = r1 - __uint_as_float(m);
    hi = b >> 16;
    mid = m >> 16;
    lo = __float_as_uint(r2) >> 16;
}

// Round-to-nearest bf16 of x and the remainder x - bf16(x) (exact in FP32).
__device__ __forceinline__ uint16_t bf16_split(float x, float &rest) {
    const uint32_t b = __float_as_uint(x);
    const uint32_t r = b + 0x7FFFu + ((b >> 16) & 1u);  // round to nearest even (finite x)
    const uint32_t h = r & 0xFFFF0000u;
    rest = x - __uint_as_float(h);
    return uint16_t(h >> 16);
}

}  // namespace nqes
