// Device pcg64 — the reference's per-chain random stream, draw for draw.
//
// pcg64 is pcg_engines::setseq_xsl_rr_128_64 (code/pcg_random.h:1778,1871):
// 128-bit state, multiplier 0x2360ED051FC65DA4_4385DF649FCCF645, increment
// 0x5851F42D4C957F2D_14057B7EF767814F (code/pcg_random.h:161-164). The
// single-argument constructor sets state = bump(seed + inc)
// (code/pcg_random.h:484-488); every draw advances first and outputs the new
// state, because output_previous = (sizeof(itype) <= 8) is false for 128 bits
// (code/pcg_random.h:773-780). The output is XSL-RR: rotr(hi ^ lo, hi >> 58)
// (code/pcg_random.h:1060-1083).
//
// The reference draws through libstdc++: uniform_real_distribution<double>(0,1)
// and bernoulli_distribution(0.5) each consume one 64-bit output x and form
// u = double(x) * 2^-64 (generate_canonical with one term, clamped to
// nextafter(1, 0) if it rounds to 1); Bernoulli is u < 0.5
// (libstdc++ bits/random.tcc generate_canonical, bits/random.h
// bernoulli_distribution::operator()).
#pragma once
#include <cstdint>

namespace nqes {

struct Pcg64 {
    uint64_t lo, hi;
};

constexpr uint64_t kPcgMulHi = 2549297995355413924ULL;
constexpr uint64_t kPcgMulLo = 4865540595714422341ULL;
constexpr uint64_t kPcgIncHi = 6364136223846793005ULL;
constexpr uint64_t kPcgIncLo = 1442695040888963407ULL;

// state = state * mul + inc  (mod 2^128)
__host__ __device__ __forceinline__ void pcg_bump(Pcg64 &g) {
#ifdef __CUDA_ARCH__
    uint64_t plo = g.lo * kPcgMulLo;
    uint64_t phi = __umul64hi(g.lo, kPcgMulLo) + g.lo * kPcgMulHi + g.hi * kPcgMulLo;
#else
    unsigned __int128 p = (unsigned __int128)g.lo * kPcgMulLo;
    uint64_t plo = (uint64_t)p;
    uint64_t phi = (uint64_t)(p >> 64) + g.lo * kPcgMulHi + g.hi * kPcgMulLo;
#endif
    uint64_t lo = plo + kPcgIncLo;
    uint64_t carry = lo < plo ? 1u : 0u;
    g.lo = lo;
    g.hi = phi + kPcgIncHi + carry;
}

__host__ __device__ __forceinline__ Pcg64 pcg_seed(uint64_t seed) {
    Pcg64 g;
    g.lo = seed + kPcgIncLo;
    g.hi = kPcgIncHi + (g.lo < seed ? 1u : 0u);
    pcg_bump(g);
    return g;
}

__host__ __device__ __forceinline__ uint64_t pcg_next(Pcg64 &g) {
    pcg_bump(g);
    uint64_t x = g.hi ^ g.lo;
    unsigned rot = unsigned(g.hi >> 58);
    return (x >> rot) | (x << ((64u - rot) & 63u));
}

// libstdc++ generate_canonical<double, 53> of one 64-bit engine output.
__device__ __forceinline__ double pcg_u01(uint64_t x) {
    double u = __ull2double_rn(x) * 0x1p-64;
    return u >= 1.0 ? 0x1.fffffffffffffp-1 : u;
}

// The same value built with integer instructions only: round x to 53
// significant bits (to nearest, ties to even), scale by 2^-64 through the
// exponent field, clamp 1.0 to the largest double below it. Returns the IEEE
// bit pattern. On GB300 this keeps the conversion off the FP64 pipe.
__host__ __device__ __forceinline__ uint64_t pcg_u01_bits(uint64_t x) {
    if (x == 0) return 0;
#ifdef __CUDA_ARCH__
    const int lz = __clzll(static_cast<long long>(x));
#else
    const int lz = __builtin_clzll(x);
#endif
    const uint64_t y = x << lz;          // leading one at bit 63
    uint64_t m = y >> 11;                // 53 significant bits
    const uint64_t rem = y & 0x7FFULL;   // the 11 bits rounded away
    if (rem > 0x400ULL || (rem == 0x400ULL && (m & 1ULL))) m++;
    int e = 63 - lz - 64;                // x * 2^-64 = 1.f * 2^e before rounding
    if (m >> 53) {                       // rounding carried into a new bit
        m >>= 1;
        e++;
    }
    if (e >= 0) return 0x3FEFFFFFFFFFFFFFULL;  // rounded to 1.0: clamp below 1
    return (uint64_t(e + 1023) << 52) | (m & 0xFFFFFFFFFFFFFULL);
}
__device__ __forceinline__ double pcg_uniform(Pcg64 &g) { return pcg_u01(pcg_next(g)); }

// bernoulli_distribution(0.5): true (spin down) iff u < 0.5.
__device__ __forceinline__ bool pcg_bernoulli_half(Pcg64 &g) { return pcg_uniform(g) < 0.5; }

}  // namespace nqes
