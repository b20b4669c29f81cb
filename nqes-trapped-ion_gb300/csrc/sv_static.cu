// S·v that allocates nothing: nqes_apply_S_static.
//
// Some callers cannot call cudaMalloc: code that runs while a CUDA graph is
// being captured on the calling thread, hosts that have handed all device
// memory to their own pool allocator and forbid allocations from plugins, and
// latency-critical loops that cannot afford the device-wide synchronisation
// cudaMalloc/cudaFree imply. For them this entry point computes the S·v of the
// matrix-free stochastic-reconfiguration operator on buffers the caller
// already owns, and keeps its own intermediates in a fixed device array that
// is part of the library image.
//
// The scratch is kScratchBytes (16 MiB) of file-scope __device__ memory. Every
// GPU that loads libnqes holds it until the process exits. Host code cannot
// pass the array's name to a kernel (in host code it is only a stand-in, not a
// device address), so the first call on each device looks its address up with
// cudaGetSymbolAddress while that device is current and caches it. The device
// is the one `stream` belongs to (the current device for the NULL stream); the
// call makes it current while it runs. Make the first call on each device
// before any stream capture begins. Every call shares the one array
// and calls that overlap on the GPU race on it, so serialise them (one stream,
// or events). Each call writes every scratch element before reading it, so
// nothing has to start at zero and the previous call's leftovers are harmless.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/nqes.h"
#include "nqes_internal.h"

namespace nqes {
void set_global_error(const std::string &msg);
}

namespace {

using nqes::cplx;

constexpr size_t kScratchBytes = size_t(16) << 20;
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_sv_scratch[kScratchBytes];

std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_sv_scratch on device `dev`, which must be current
// (looked up once per device).
cudaError_t scratch_address(int dev, void **out) {
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sv_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return cudaSuccess;
}

template <class S> __device__ __forceinline__ S load(const S *p) { return *p; }

// u_s = sum_p O_sp v_p, one warp per row.
template <class S> __global__ void k_rows(long long ns, long long P, const S *O, const S *v, S *u) {
    const long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= ns) return;
    const S *r = O + row * P;
    S acc = nqes::zero<S>();
    for (long long p = lane; p < P; p += 32) acc = nqes::mad(r[p], v[p], acc);
    acc = nqes::warp_sum(acc);
    if (lane == 0) u[row] = acc;
}

// ypart[c][p] = sum over rows of chunk c of conj(O_sp) u_s.
template <class S>
__global__ void k_cols(long long ns, long long P, int chunks, const S *O, const S *u, S *ypart) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (p >= P) return;
    const long long s0 = ns * c / chunks, s1 = ns * (c + 1) / chunks;
    S acc = nqes::zero<S>();
    for (long long s = s0; s < s1; s++) acc = nqes::cmad(O[s * P + p], u[s], acc);
    ypart[c * P + p] = acc;
}

// ovpart[b] = sum over block b of o_p v_p.
template <class S> __global__ void k_ov(long long P, const S *o, const S *v, S *ovpart) {
    __shared__ S sh[kThreads / 32];
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    S t = p < P ? o[p] * v[p] : nqes::zero<S>();
    t = nqes::warp_sum(t);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        S s = nqes::zero<S>();
        for (int w = 0; w < kThreads / 32; w++) s = s + sh[w];
        ovpart[blockIdx.x] = s;
    }
}

// out_p = (sum_c ypart[c][p]) / Ns + skk_p v_p - (o·v) conj(o_p)
template <class S>
__global__ void k_finish(long long ns, long long P, int chunks, int nb, const S *ypart, const S *ovpart, const S *o,
                         const S *skk, const S *v, S *out) {
    __shared__ S ov_s;
    if (threadIdx.x < 32) {
        S s = nqes::zero<S>();
        for (int b = threadIdx.x; b < nb; b += 32) s = s + ovpart[b];
        s = nqes::warp_sum(s);
        if (threadIdx.x == 0) ov_s = s;
    }
    __syncthreads();
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= P) return;
    S y = nqes::zero<S>();
    for (int c = 0; c < chunks; c++) y = y + ypart[c * P + p];
    y = y * (1.0 / double(ns));
    y = nqes::mad(skk[p], v[p], y);
    out[p] = y - ov_s * nqes::conj(o[p]);
}

template <class S>
int run(const S *O, const S *o, const S *skk, const S *v, S *out, long long ns, long long P, int dev,
        cudaStream_t st) {
    const size_t cap = kScratchBytes / sizeof(S);
    // scratch: u[ns] | ovpart[nb] | ypart[chunks * P]; each size is checked
    // against the capacity before any sum is formed, so nothing wraps
    const long long nb = P <= (long long)cap ? (P + kThreads - 1) / kThreads : 0;
    const bool fits = ns <= (long long)cap && P <= (long long)cap && size_t(ns) + size_t(nb) + size_t(P) <= cap;
    if (!fits) {
        const double need = (double(ns) + double(P) / kThreads + double(P)) * sizeof(S);
        nqes::set_global_error("nqes_apply_S_static: " + std::to_string(need) +
                               " bytes of scratch needed for n_samples=" + std::to_string(ns) +
                               ", n_params=" + std::to_string(P) + "; the static scratch holds " +
                               std::to_string(kScratchBytes) + " bytes");
        return NQES_ERR_INVALID;
    }
    int chunks = int((cap - size_t(ns) - size_t(nb)) / size_t(P));
    chunks = chunks > 32 ? 32 : chunks;
    const long long by_rows = (ns + 255) / 256;
    if (chunks > by_rows) chunks = int(by_rows < 1 ? 1 : by_rows);
    void *base = nullptr;
    cudaError_t e = scratch_address(dev, &base);
    if (e != cudaSuccess) {
        nqes::set_global_error(std::string("nqes_apply_S_static: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        return NQES_ERR_CUDA;
    }
    S *u = static_cast<S *>(base);
    S *ovpart = u + ns;
    S *ypart = ovpart + nb;
    const long long rows_per_block = kThreads / 32;
    k_rows<S><<<unsigned((ns + rows_per_block - 1) / rows_per_block), kThreads, 0, st>>>(ns, P, O, v, u);
    k_cols<S><<<dim3(unsigned(nb), unsigned(chunks)), kThreads, 0, st>>>(ns, P, chunks, O, u, ypart);
    k_ov<S><<<unsigned(nb), kThreads, 0, st>>>(P, o, v, ovpart);
    k_finish<S><<<unsigned(nb), kThreads, 0, st>>>(ns, P, chunks, int(nb), ypart, ovpart, o, skk, v, out);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        nqes::set_global_error(std::string("nqes_apply_S_static: launch: ") + cudaGetErrorString(e));
        return NQES_ERR_CUDA;
    }
    return NQES_OK;
}

}  // namespace

extern "C" int nqes_apply_S_static(const double *O, const double *o, const double *skk, const double *v, double *out,
                                   int64_t n_samples, int64_t n_params, int complex_arith, void *stream) {
    if (!O || !o || !skk || !v || !out || n_samples < 1 || n_params < 1 ||
        (complex_arith != 0 && complex_arith != 1)) {
        nqes::set_global_error("nqes_apply_S_static: null pointer, non-positive size or complex_arith not 0/1");
        return NQES_ERR_INVALID;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // The work runs on the stream's device, and the scratch address looked up
    // is that device's: make it current for the call, then restore the caller's.
    int cur = 0, dev = 0;
    cudaError_t e = cudaGetDevice(&cur);
    if (e == cudaSuccess) e = st ? cudaStreamGetDevice(st, &dev) : cudaGetDevice(&dev);
    if (e == cudaSuccess && dev != cur) e = cudaSetDevice(dev);
    if (e != cudaSuccess) {
        nqes::set_global_error(std::string("nqes_apply_S_static: device of the stream: ") + cudaGetErrorString(e));
        return NQES_ERR_CUDA;
    }
    const int rc = complex_arith
                       ? run<cplx>(reinterpret_cast<const cplx *>(O), reinterpret_cast<const cplx *>(o),
                                   reinterpret_cast<const cplx *>(skk), reinterpret_cast<const cplx *>(v),
                                   reinterpret_cast<cplx *>(out), n_samples, n_params, dev, st)
                       : run<double>(O, o, skk, v, out, n_samples, n_params, dev, st);
    if (dev != cur) cudaSetDevice(cur);
    return rc;
}
