// CPU oracle — test infrastructure only. Nothing in the product links this file.
//
// Restatement of the reference's random-number generator: `pcg64`, i.e.
// pcg_engines::setseq_xsl_rr_128_64 (code/pcg_random.h:1871), a 128-bit LCG
// with the default 128-bit multiplier and increment (code/pcg_random.h:161-164),
// constructed from a single seed value (code/pcg_random.h:484-488: state =
// bump(seed + increment)). Each draw first advances the state and then emits
// the XSL-RR output of the *new* state: setseq_base sets output_previous =
// (sizeof(itype) <= 8), which is false for the 128-bit state
// (code/pcg_random.h:773-780, 431-437, 1060-1083).
//
// The class satisfies the C++ UniformRandomBitGenerator requirements, so the
// libstdc++ distributions the reference uses (bernoulli_distribution,
// uniform_real_distribution<double>, normal_distribution<double>) run on it
// unchanged, exactly as they do in code/rbm.cc:103,264,535.
#pragma once
#include <cstdint>

namespace nqes_oracle {

class Pcg64 {
public:
    using result_type = uint64_t;
    using u128 = __uint128_t;

    static constexpr u128 kMult =
        (u128(2549297995355413924ULL) << 64) + u128(4865540595714422341ULL);
    static constexpr u128 kInc =
        (u128(6364136223846793005ULL) << 64) + u128(1442695040888963407ULL);

    // pcg64(seed): the 64-bit seed is widened to 128 bits, then bumped once.
    explicit Pcg64(uint64_t seed) : state_((u128(seed) + kInc) * kMult + kInc) {}

    static constexpr result_type min() { return 0; }
    static constexpr result_type max() { return ~uint64_t(0); }

    result_type operator()() {
        state_ = state_ * kMult + kInc;
        uint64_t hi = uint64_t(state_ >> 64), lo = uint64_t(state_);
        unsigned rot = unsigned(hi >> 58);          // top 6 bits of the state
        uint64_t x = hi ^ lo;                        // xorshift-low by 64
        return (x >> rot) | (x << ((64u - rot) & 63u));
    }

    u128 state() const { return state_; }

private:
    u128 state_;
};

}  // namespace nqes_oracle
