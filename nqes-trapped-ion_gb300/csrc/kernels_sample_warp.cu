// Decision-warp sampler: instantiations for K = 1, 2 and the host-side
// launch, occupancy and table functions (K = 3, 4 are instantiated in
// kernels_sample_warp_k34.cu). The kernels are in sample_warp.cuh.
#include "sample_warp.cuh"

namespace nqes {

// K = 3, 4 instances, from kernels_sample_warp_k34.cu
void *dw_kernel_k34(int K, int U);

namespace {

using DwKernel = void (*)(const MixedArgs);
template <int K> DwKernel dw_kernel_u(int U) {
    switch (U) {
    case 1: return k_sample_dw<K, 1>;
    case 2: return k_sample_dw<K, 2>;
    case 4: return k_sample_dw<K, 4>;
    case 8: return k_sample_dw<K, 8>;
    case 16: return k_sample_dw<K, 16>;
    case 32: return k_sample_dw<K, 32>;
    default: return nullptr;
    }
}
DwKernel dw_kernel(int K, int U) {
    switch (K) {
    case 1: return dw_kernel_u<1>(U);
    case 2: return dw_kernel_u<2>(U);
    default: return reinterpret_cast<DwKernel>(dw_kernel_k34(K, U));
    }
}

}  // namespace

// Units per lane of the decision-warp form for (M, K): G = largest power of two
// <= 32/K lanes per RBM, U = M/G rounded up to a power of two; 0 if U > 32.
int dw_units(const Shape &sh, int *G_out) {
    int G = 32;
    while (G * sh.K > 32) G >>= 1;
    int U = 1;
    while (U * G < sh.M) U <<= 1;
    if (G_out) *G_out = G;
    return U <= 32 ? U : 0;
}

size_t dw_smem_bytes(const Shape &sh, int MP, bool staged, bool out64) {
    return dsmem_bytes(sh.N, MP, sh.K, staged, out64);
}

cudaError_t prepare_sample_dw(const Shape &sh, int MP) {
    int G = 0;
    const DwKernel fn = dw_kernel(sh.K, dw_units(sh, &G));
    if (!fn || G * dw_units(sh, nullptr) != MP) return cudaErrorInvalidConfiguration;
    return allow_max_dynamic_smem(reinterpret_cast<const void *>(fn));
}

cudaError_t dw_occupancy(const Shape &sh, int threads, size_t smem, int *blocks_per_sm) {
    const DwKernel fn = dw_kernel(sh.K, dw_units(sh, nullptr));
    if (!fn) return cudaErrorInvalidConfiguration;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, reinterpret_cast<const void *>(fn), threads,
                                                         smem);
}

cudaError_t launch_sample_dw(const MixedArgs &a, int warps, cudaStream_t st) {
    const size_t smem = dsmem_bytes(a.sh.N, a.MP, a.sh.K, a.stage != 0, a.out64 != 0 || a.e64 != 0);
    const DwKernel fn = dw_kernel(a.sh.K, a.U);
    if (!fn || warps < 1 || warps > 8 || a.sh.NW > 2 || a.G * a.U != a.MP) return cudaErrorInvalidConfiguration;
    fn<<<a.chains, 32 * warps, smem, st>>>(a);
    return cudaGetLastError();
}

namespace {
__global__ void k_exp_table(double *tab) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < kExpTabN) tab[n] = exp(-double(n) / 64.0);
}
}  // namespace

cudaError_t launch_exp_table(double *tab, cudaStream_t st) {
    k_exp_table<<<(kExpTabN + 255) / 256, 256, 0, st>>>(tab);
    return cudaGetLastError();
}

cudaError_t launch_tables_dw(const Shape &sh, int MP, const cplx *b, const cplx *w, float *cp, float *spp, float *whp,
                             float *wlp, float *bh, float *bl, float *bnd, float *cpl, float *spl, cudaStream_t st) {
    const size_t n = size_t(sh.K) * sh.N * MP;
    const int blocks = int(std::min<size_t>((n + 255) / 256, 4096));
    const cudaError_t e = cudaMemsetAsync(bnd + 4 * size_t(sh.K) * sh.N, 0, sizeof(float) * sh.K, st);
    if (e != cudaSuccess) return e;
    k_tables_dw<<<blocks, 256, 0, st>>>(sh, MP, b, w, cp, spp, whp, wlp, bh, bl, reinterpret_cast<float4 *>(bnd), cpl,
                                        spl);
    return cudaGetLastError();
}

}  // namespace nqes
