// S·v over the dense FP64 log-derivatives in ONE read of O, off the FP64 pipe.
//
// The S·v of code/rbm.cc:660-683 over the stored O (real arithmetic, the
// FP64 and certified forms) is y = O^T (O v) plus diagonal and rank-one terms
// that the Lanczos kernels add. Two separate passes (u = O v, then O^T u)
// read the Ns × P matrix twice and run two FP64 FMAs per entry on a part whose
// FP64 pipe retires about two FMAs per SM per clock: 0.41 ms at N32 M64 K2.
//
// Here a persistent CTA per SM owns a contiguous range of rows and streams
// them through shared memory in groups of G rows (as many as two buffers of
// shared memory hold, at most 16), double-buffered by bulk copies
// (cp.async.bulk on an mbarrier, bounded waits). For each staged group
//   pass 1: u_r = O_r . v for the group's rows, block-wide, and
//   pass 2: y_p += O_rp u_r into the CTA's partial of O^T u (registers),
// both from shared memory, so O leaves HBM once per S·v. The arithmetic is
// double-float on the FP32 pipe: each FP64 entry d is split exactly-enough
// into hi + lo floats by integer operations (hi = d cut to 24 significant
// bits, lo = the remaining 29 bits rounded to 24: |d - hi - lo| <= 2^-48 |d|,
// nqes_math.cuh), products are formed with their FMA error terms, sums are
// TwoSum-compensated. The certified sampler stores O already split (the
// pairs in the FP64 slots), which saves the split here; O written as FP64
// (the FP64 sampler) is split in shared memory on its first read.
// The relative error of u and of the partials against FP64 sums of the same
// terms is a few 2^-48 per term of sum |O v| (about 1e-14 at these sizes),
// inside the 1e-12 parity bound. Entries below 2^-126 in magnitude count as
// zero (absolute error under 1e-38); an entry of O of magnitude 2^127 or
// more, or a non-finite one, sets kErrNonFinite.
//
// Each CTA writes its partial y (converted to FP64) to ypart[cta]; the
// Lanczos epilogue sums the partials over CTAs in a fixed order, so results
// do not depend on timing.
#include <algorithm>

#include "nqes_internal.h"
#include "tma_stage.cuh"

namespace nqes {
namespace {

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

struct FusedSvArgs {
    int Ns, P, G;
    int o_split;  // O already stored as (hi, lo) pairs
    const double *O, *v;
    double *ypart;  // gridDim.x × P
    int *err;
    const int *guard;
};

constexpr int kFsMaxThreads = 1024;
constexpr int kFsMaxWarps = kFsMaxThreads / 32;

// Block: T = blockDim.x threads (a multiple of 32, T C >= P); thread t owns
// columns p = t + c T (c < C), holding v's split and its partial of O^T u for
// them in registers. Rows of a staged group are walked one at a time, so no
// per-row state lives in registers.
// Dynamic shared memory of a launch: two staged groups of G rows, the
// per-warp partials of u, u itself, two mbarriers.
__host__ __device__ inline size_t fused_smem(int P, int G) {
    return size_t(2) * G * P * sizeof(double) + (size_t(G) * kFsMaxWarps + G + 1) * sizeof(float2) +
           2 * sizeof(uint64_t);
}

template <int C, int MaxT, bool PRE>
__global__ void __launch_bounds__(MaxT, 1) k_sv_fused(FusedSvArgs a) {
    extern __shared__ __align__(16) unsigned char fs_smem[];
    if (loop_guard_off(a.guard)) return;
    const int P = a.P, G = a.G, T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = T >> 5;
    if (!dyn_smem_covers(fused_smem(P, G)) || nw > kFsMaxWarps || T * C < P) {
        if (tid == 0) atomicOr(a.err, kErrLaunch);
        return;
    }
    double *buf0 = reinterpret_cast<double *>(fs_smem);
    double *buf1 = buf0 + size_t(G) * P;
    float2 *red = reinterpret_cast<float2 *>(buf1 + size_t(G) * P);  // [G][warps]
    float2 *us = red + size_t(G) * kFsMaxWarps;                       // [G]
    uint64_t *mbar = reinterpret_cast<uint64_t *>(us + G + (G & 1));  // [2], 8-byte aligned
    const int r0 = int(int64_t(a.Ns) * blockIdx.x / gridDim.x), r1 = int(int64_t(a.Ns) * (blockIdx.x + 1) / gridDim.x);
    const int ngroups = (r1 - r0 + G - 1) / G;

    float vh[C], vl[C], yh[C], yl[C];
    bool range_ok = true;  // of the O entries (v is not checked: a solve that never starts has v = 0/0)
#pragma unroll
    for (int c = 0; c < C; c++) {
        const int p = tid + c * T;
        vh[c] = vl[c] = yh[c] = yl[c] = 0.f;
        if (p < P) df_split(a.v[p], vh[c], vl[c]);
    }
    auto issue = [&](int g) {  // thread 0: group g into buffer g & 1
        const int rs = r0 + g * G, nr = min(G, r1 - rs);
        const unsigned bytes = unsigned(size_t(nr) * P * sizeof(double));
        uint64_t *mb = &mbar[g & 1];
        mbar_expect_tx(mb, bytes);
        bulk_g2s(g & 1 ? buf1 : buf0, a.O + size_t(rs) * P, bytes, mb);
    };
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
    }
    __syncthreads();
    if (tid == 0) {
        if (ngroups > 0) issue(0);
        if (ngroups > 1) issue(1);
    }
    bool timed_out = false;
    int g = 0;
    for (; g < ngroups; g++) {
        double *buf = g & 1 ? buf1 : buf0;
        const int nr = min(G, r1 - (r0 + g * G));
        const bool ok = mbar_wait(&mbar[g & 1], unsigned(g >> 1) & 1u);
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        // pass 1, row by row: split the staged entries in place (each thread
        // its own columns, read back only by itself), the row's dot product
        // with v, its warp sum to red[r][warp]
        for (int r = 0; r < nr; r++) {
            double *row = buf + size_t(r) * P;
            // two accumulators (even and odd columns) for two independent chains
            float h = 0.f, l = 0.f, h2 = 0.f, l2 = 0.f;
#pragma unroll
            for (int c = 0; c < C; c++) {
                const int p = tid + c * T;
                if (p < P) {
                    float oh, ol;
                    if (PRE) {  // split when it was written
                        const float2 o = *reinterpret_cast<const float2 *>(row + p);
                        oh = o.x;
                        ol = o.y;
                    } else {
                        range_ok &= df_split(row[p], oh, ol);
                        *reinterpret_cast<float2 *>(row + p) = make_float2(oh, ol);
                    }
                    if (c & 1)
                        df_fma(h2, l2, oh, ol, vh[c], vl[c]);
                    else
                        df_fma(h, l, oh, ol, vh[c], vl[c]);
                }
            }
            df_acc(h, l, h2, l2);
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) {
                const float oh = __shfl_down_sync(0xffffffffu, h, off), ol = __shfl_down_sync(0xffffffffu, l, off);
                df_acc(h, l, oh, ol);
            }
            if (lane == 0) red[r * kFsMaxWarps + warp] = make_float2(h, l);
        }
        __syncthreads();
        // u_r: the warps' sums in warp order, one warp per row
        for (int r = warp; r < nr; r += nw) {
            float h = 0.f, l = 0.f;
            if (lane == 0)
                for (int w = 0; w < nw; w++) df_acc(h, l, red[r * kFsMaxWarps + w].x, red[r * kFsMaxWarps + w].y);
            if (lane == 0) us[r] = make_float2(h, l);
        }
        __syncthreads();
        // pass 2: y_p += O_rp u_r over the group's rows
        for (int r = 0; r < nr; r++) {
            const float2 u = us[r];
            const double *row = buf + size_t(r) * P;
#pragma unroll
            for (int c = 0; c < C; c++) {
                const int p = tid + c * T;
                if (p < P) {
                    const float2 o = *reinterpret_cast<const float2 *>(row + p);
                    df_fma(yh[c], yl[c], o.x, o.y, u.x, u.y);
                }
            }
        }
        // every thread is done with buf (and with us); its in-place splits
        // (generic proxy) are ordered before the next bulk copy (async proxy)
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0 && g + 2 < ngroups) issue(g + 2);
    }
    if (timed_out) {
        if (tid == 0) {
            atomicOr(a.err, kErrTimeout);
            // wait (bounded) for the copies still in flight into this CTA's buffers
            for (int q = g; q < min(g + 2, ngroups); q++) mbar_wait(&mbar[q & 1], unsigned(q >> 1) & 1u);
        }
        return;
    }
    if (!range_ok) atomicOr(a.err, kErrNonFinite);
#pragma unroll
    for (int c = 0; c < C; c++) {
        const int p = tid + c * T;
        if (p < P) a.ypart[size_t(blockIdx.x) * P + p] = double(yh[c]) + double(yl[c]);
    }
}

// Columns per thread C and threads per block T (whole warps, T C >= P): the
// fewest columns whose block fits its register budget: C = 1, 2, 4 with up to
// 1024 threads (64 registers), 8 with up to 768, 16 with up to 512.
constexpr int kFsShapes[5][2] = {{1, 1024}, {2, 1024}, {4, 1024}, {8, 768}, {16, 512}};
bool fused_shape(int P, int *C, int *T) {
    for (const auto &sh : kFsShapes) {
        const int t = 32 * ((P + 32 * sh[0] - 1) / (32 * sh[0]));
        if (t <= sh[1]) {
            *C = sh[0];
            *T = t;
            return true;
        }
    }
    return false;
}

template <bool PRE, class F> cudaError_t fused_dispatch_p(int C, F &&f) {
    switch (C) {
    case 1: return f(k_sv_fused<1, 1024, PRE>);
    case 2: return f(k_sv_fused<2, 1024, PRE>);
    case 4: return f(k_sv_fused<4, 1024, PRE>);
    case 8: return f(k_sv_fused<8, 768, PRE>);
    default: return f(k_sv_fused<16, 512, PRE>);
    }
}
template <class F> cudaError_t fused_dispatch(int C, F &&f, bool pre = false) {
    return pre ? fused_dispatch_p<true>(C, f) : fused_dispatch_p<false>(C, f);
}

constexpr int kFsMaxG = 16;

}  // namespace

cudaError_t prepare_sv_fused(int P) {
    int C, T;
    if (!fused_shape(P, &C, &T)) return cudaErrorInvalidValue;
    auto set = [](auto fn) { return allow_max_dynamic_smem(reinterpret_cast<const void *>(fn)); };
    const cudaError_t e = fused_dispatch(C, set, false);
    return e != cudaSuccess ? e : fused_dispatch(C, set, true);
}

// Rows per staged group G and the grid: the G that keeps the most threads
// resident per SM (blocks per SM from the occupancy calculator, which counts
// the two buffers of G rows), the largest such G (fewer barriers per row);
// the grid fills every SM with that many blocks.
bool sv_fused_plan(int Ns, int P, int *G_out, int *ctas_out) {
    int C, T;
    if (P % 2 || Ns < 1 || !fused_shape(P, &C, &T)) return false;  // rows 16-byte aligned; columns in registers
    int dev = 0, sms = 152, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (prepare_sv_fused(P) != cudaSuccess) return false;
    int best_G = 0, best_blocks = 0, best_threads = 0;
    for (int G = 1; G <= kFsMaxG; G++) {
        const size_t smem = fused_smem(P, G);
        if (smem > size_t(optin) - 1024) break;
        int blocks = 0;
        const cudaError_t e = fused_dispatch(C, [&](auto fn) {
            return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, T, smem);
        });
        if (e != cudaSuccess || blocks < 1) break;
        const int threads = std::min(blocks * T, 2048);
        if (threads >= best_threads) {
            best_threads = threads;
            best_G = G;
            best_blocks = blocks;
        }
    }
    if (!best_G) return false;
    *G_out = best_G;
    *ctas_out = std::max(1, std::min(sms * best_blocks, (Ns + best_G - 1) / best_G));
    return true;
}

cudaError_t launch_sv_fused(int Ns, int P, int G, int ctas, const double *O, const double *v, double *ypart, int *err,
                            const int *guard, cudaStream_t st, bool o_split) {
    FusedSvArgs a{Ns, P, G, o_split ? 1 : 0, O, v, ypart, err, guard};
    const size_t smem = fused_smem(P, G);
    int C, T;
    if (!fused_shape(P, &C, &T)) return cudaErrorInvalidValue;
    return fused_dispatch(
        C,
        [&](auto fn) {
            fn<<<ctas, T, smem, st>>>(a);
            return cudaGetLastError();
        },
        o_split);
}

}  // namespace nqes
