// Decision-warp sampler: instantiations for K = 3, 4 (a separate translation
// unit so that the instances compile in parallel).
#include <type_traits>

#include "sample_warp.cuh"

namespace nqes {

void *dw_kernel_k34(int K, int U) {
    auto pick = [&](auto k) -> void * {
        constexpr int KK = decltype(k)::value;
        switch (U) {
        case 1: return reinterpret_cast<void *>(k_sample_dw<KK, 1>);
        case 2: return reinterpret_cast<void *>(k_sample_dw<KK, 2>);
        case 4: return reinterpret_cast<void *>(k_sample_dw<KK, 4>);
        case 8: return reinterpret_cast<void *>(k_sample_dw<KK, 8>);
        case 16: return reinterpret_cast<void *>(k_sample_dw<KK, 16>);
        case 32: return reinterpret_cast<void *>(k_sample_dw<KK, 32>);
        default: return nullptr;
        }
    };
    if (K == 3) return pick(std::integral_constant<int, 3>{});
    if (K == 4) return pick(std::integral_constant<int, 4>{});
    return nullptr;
}

}  // namespace nqes
