// S·v over the dense FP64 log-derivatives in ONE read of O, off the FP64 pipe.
//
// The S·v of code/rbm.cc:660-683 over the stored O (real arithmetic, the
// FP64 and certified forms) is y = O^T (O v) plus diagonal and rank-one terms
// that the Lanczos kernels add. Two separate passes (u = O v, then O^T u)
// read the Ns × P matrix twice and run two FP64 FMAs per entry on a part whose
// FP64 pipe retires about two FMAs per SM per clock: 0.41 ms at N32 M64 K2.
//
// Here a persistent CTA per SM owns a contiguous range of rows and streams
// them through shared memory in groups of G rows, NB groups deep (a ring of
// buffers, each filled by bulk copies (cp.async.bulk, one per row) on its own mbarrier,
// bounded waits), so that up to NB - 1 groups are in flight while one is
// used. For each staged group
//   pass 1: u_r = O_r . v, rows taken in pairs: each thread's two partial
//           dots, then one butterfly over the warp for both rows (the first
//           exchange trades one row for the other, so the pair costs five
//           exchanges, not ten), the warps' sums to shared memory;
//   pass 2: every warp sums the warps' partials of a pair of rows (again one
//           butterfly), then y_p += O_rp u_r into the CTA's partial of O^T u
//           (registers),
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

constexpr int kFsMaxThreads = 1024;
constexpr int kFsMaxWarps = kFsMaxThreads / 32;
constexpr int kFsMaxG = 16;  // rows per group
constexpr int kFsMaxNB = 4;  // groups in the ring

struct FusedSvArgs {
    int Ns, P, G, NB;
    int o_split;  // O already stored as (hi, lo) pairs
    const double *O, *v;
    double *ypart;  // gridDim.x × P
    int *err;
    const int *guard;
};

// Dynamic shared memory of a launch: NB groups of G rows of Q >= P entries
// (each row padded with zeros to the block's T C columns), the warps'
// partials of the group's u (float2 [G][warps]), NB mbarriers.
__host__ __device__ inline size_t fused_smem(int Q, int G, int NB) {
    return size_t(NB) * G * Q * sizeof(double) + size_t(G) * kFsMaxWarps * sizeof(float2) +
           size_t(NB) * sizeof(uint64_t);
}

// The double-float pairs (h0, l0) and (h1, l1) summed over the warp in a
// fixed order: the first exchange (lanes i and i + 16) sends the row a lane
// does not keep, the next four reduce the kept row within each half. Returns
// the first row's sum in lane 0 and the second's in lane 16 (the other lanes
// hold the same sums in other orders).
__device__ __forceinline__ void warp_sum_pair(float &h, float &l, float h0, float l0, float h1, float l1) {
    const bool upper = (threadIdx.x & 16) != 0;
    h = upper ? h1 : h0;
    l = upper ? l1 : l0;
    const float sh = upper ? h0 : h1, sl = upper ? l0 : l1;
    df_acc(h, l, __shfl_xor_sync(0xffffffffu, sh, 16), __shfl_xor_sync(0xffffffffu, sl, 16));
#pragma unroll
    for (int off = 8; off > 0; off >>= 1)
        df_acc(h, l, __shfl_xor_sync(0xffffffffu, h, off), __shfl_xor_sync(0xffffffffu, l, off));
}

// Block: T = blockDim.x threads (a multiple of 32, Q = T C >= P); thread t
// owns the C consecutive columns p = t C + c (c < C), holding v's split and
// its partial of O^T u for them in registers. Rows sit in shared memory at
// stride Q with the columns P..Q-1 zero (v is zero there too), so the inner
// loops carry no column test and address a thread's entries at fixed offsets
// from its row pointer; with C odd, the 8-byte entries of a half-warp fall in
// distinct bank pairs.
template <int C, int MaxT, bool PRE>
__global__ void __launch_bounds__(MaxT, 1) k_sv_fused(FusedSvArgs a) {
    extern __shared__ __align__(16) unsigned char fs_smem[];
    if (loop_guard_off(a.guard)) return;
    const int P = a.P, G = a.G, NB = a.NB, T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5,
              nw = T >> 5, Q = T * C;
    if (!dyn_smem_covers(fused_smem(Q, G, NB)) || nw > kFsMaxWarps || Q < P || G > kFsMaxG || NB < 2 ||
        NB > kFsMaxNB) {
        if (tid == 0) atomicOr(a.err, kErrLaunch);
        return;
    }
    double *bufs = reinterpret_cast<double *>(fs_smem);                   // [NB][G][Q]
    float2 *red = reinterpret_cast<float2 *>(bufs + size_t(NB) * G * Q);  // [G][kFsMaxWarps]
    uint64_t *mbar = reinterpret_cast<uint64_t *>(red + size_t(G) * kFsMaxWarps);  // [NB]
    const int r0 = int(int64_t(a.Ns) * blockIdx.x / gridDim.x), r1 = int(int64_t(a.Ns) * (blockIdx.x + 1) / gridDim.x);
    const int ngroups = (r1 - r0 + G - 1) / G;
    const int p0 = tid * C;  // this thread's first column

    float vh[C], vl[C], yh[C], yl[C];
    bool range_ok = true;  // of the O entries (v is not checked: a solve that never starts has v = 0/0)
#pragma unroll
    for (int c = 0; c < C; c++) {
        vh[c] = vl[c] = yh[c] = yl[c] = 0.f;
        if (p0 + c < P) df_split(a.v[p0 + c], vh[c], vl[c]);
    }
    // the padding of every staged row: zero once (the copies write [0, P) only)
    const int pad = Q - P;
    for (int i = tid; i < NB * G * pad; i += T) bufs[size_t(i / pad) * Q + P + i % pad] = 0.0;
    auto issue = [&](int g) {  // thread 0: group g into ring slot g % NB, one copy per row
        const int rs = r0 + g * G, nr = min(G, r1 - rs);
        uint64_t *mb = &mbar[g % NB];
        double *dst = bufs + size_t(g % NB) * G * Q;
        mbar_expect_tx(mb, unsigned(size_t(nr) * P * sizeof(double)));
        for (int i = 0; i < nr; i++)
            bulk_g2s(dst + size_t(i) * Q, a.O + size_t(rs + i) * P, unsigned(size_t(P) * sizeof(double)), mb);
    };
    if (tid == 0)
        for (int b = 0; b < NB; b++) mbar_init(&mbar[b], 1);
    __syncthreads();
    if (tid == 0)
        for (int g = 0; g < min(NB, ngroups); g++) issue(g);

    // entry c of the thread's part of a staged row as (hi, lo); FP64 entries
    // are split in place (each thread its own columns, read back only by
    // itself in pass 2)
    auto entry = [&](double *row, int c, float &oh, float &ol) {
        if (PRE) {  // split when it was written
            const float2 o = *reinterpret_cast<const float2 *>(row + c);
            oh = o.x;
            ol = o.y;
        } else {
            range_ok &= df_split(row[c], oh, ol);
            *reinterpret_cast<float2 *>(row + c) = make_float2(oh, ol);
        }
    };

    bool timed_out = false;
    int g = 0;
    for (; g < ngroups; g++) {
        double *buf = bufs + size_t(g % NB) * G * Q;
        const int nr = min(G, r1 - (r0 + g * G));
        const bool ok = mbar_wait(&mbar[g % NB], unsigned(g / NB) & 1u);
        if (__syncthreads_or(!ok)) {
            timed_out = true;
            break;
        }
        // pass 1: rows in pairs, one chain per row; the warp's sums of rows
        // r and r + 1 to red
        for (int r = 0; r < nr; r += 2) {
            double *row0 = buf + size_t(r) * Q + p0, *row1 = row0 + Q;
            float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
            if (r + 1 < nr) {
#pragma unroll
                for (int c = 0; c < C; c++) {
                    float oh, ol, qh, ql;
                    entry(row0, c, oh, ol);
                    entry(row1, c, qh, ql);
                    df_fma(h0, l0, oh, ol, vh[c], vl[c]);
                    df_fma(h1, l1, qh, ql, vh[c], vl[c]);
                }
            } else {
#pragma unroll
                for (int c = 0; c < C; c++) {
                    float oh, ol;
                    entry(row0, c, oh, ol);
                    df_fma(h0, l0, oh, ol, vh[c], vl[c]);
                }
            }
            float h, l;
            warp_sum_pair(h, l, h0, l0, h1, l1);
            if (lane == 0) red[r * kFsMaxWarps + warp] = make_float2(h, l);
            if (lane == 16 && r + 1 < nr) red[(r + 1) * kFsMaxWarps + warp] = make_float2(h, l);
        }
        __syncthreads();
        // pass 2: per pair of rows, u from the warps' sums (every warp alike,
        // in warp order), then y_p += O_rp u_r
        for (int r = 0; r < nr; r += 2) {
            const bool two = r + 1 < nr;
            float2 s0 = make_float2(0.f, 0.f), s1 = make_float2(0.f, 0.f);
            if (lane < nw) {
                s0 = red[r * kFsMaxWarps + lane];
                if (two) s1 = red[(r + 1) * kFsMaxWarps + lane];
            }
            float h, l;
            warp_sum_pair(h, l, s0.x, s0.y, s1.x, s1.y);
            const float u0h = __shfl_sync(0xffffffffu, h, 0), u0l = __shfl_sync(0xffffffffu, l, 0);
            const float u1h = __shfl_sync(0xffffffffu, h, 16), u1l = __shfl_sync(0xffffffffu, l, 16);
            const float2 *row0 = reinterpret_cast<const float2 *>(buf + size_t(r) * Q + p0), *row1 = row0 + Q;
            if (two) {
#pragma unroll
                for (int c = 0; c < C; c++) {
                    const float2 o = row0[c], q = row1[c];
                    df_fma(yh[c], yl[c], o.x, o.y, u0h, u0l);
                    df_fma(yh[c], yl[c], q.x, q.y, u1h, u1l);
                }
            } else {
#pragma unroll
                for (int c = 0; c < C; c++) {
                    const float2 o = row0[c];
                    df_fma(yh[c], yl[c], o.x, o.y, u0h, u0l);
                }
            }
        }
        // every thread is done with the slot and with red; its in-place splits
        // (generic proxy) are ordered before the next bulk copy (async proxy)
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0 && g + NB < ngroups) issue(g + NB);
    }
    if (timed_out) {
        if (tid == 0) {
            atomicOr(a.err, kErrTimeout);
            // wait (bounded) for the copies still in flight into this CTA's ring
            for (int q = g; q < min(g + NB, ngroups); q++) mbar_wait(&mbar[q % NB], unsigned(q / NB) & 1u);
        }
        return;
    }
    if (!range_ok) atomicOr(a.err, kErrNonFinite);
#pragma unroll
    for (int c = 0; c < C; c++)
        if (p0 + c < P) a.ypart[size_t(blockIdx.x) * P + p0 + c] = double(yh[c]) + double(yl[c]);
}

// Columns per thread C and threads per block T (whole warps, T C >= P): the
// fewest columns, C odd (conflict-free shared-memory reads), whose block has
// at most the row's thread limit. Each staged row pair costs every warp two
// butterflies whatever C is, so blocks of 500 or so threads with more columns
// each beat full-size blocks once P passes 3000: at P = 4288 (N32 M64 K2),
// 0.214 ms per S·v with C = 5 (864 threads), 0.193 with 7 (640), 0.180 with 9
// (480), 0.203 with 11 (416), 0.182 with 17 (256, two blocks per SM).
constexpr int kFsShapes[6][2] = {{1, 1024}, {3, 1024}, {5, 640}, {7, 512}, {9, 512}, {17, 512}};
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
    case 3: return f(k_sv_fused<3, 1024, PRE>);
    case 5: return f(k_sv_fused<5, 640, PRE>);
    case 7: return f(k_sv_fused<7, 512, PRE>);
    case 9: return f(k_sv_fused<9, 512, PRE>);
    default: return f(k_sv_fused<17, 512, PRE>);
    }
}
template <class F> cudaError_t fused_dispatch(int C, F &&f, bool pre = false) {
    return pre ? fused_dispatch_p<true>(C, f) : fused_dispatch_p<false>(C, f);
}

}  // namespace

cudaError_t prepare_sv_fused(int P) {
    int C, T;
    if (!fused_shape(P, &C, &T)) return cudaErrorInvalidValue;
    auto set = [](auto fn) { return allow_max_dynamic_smem(reinterpret_cast<const void *>(fn)); };
    const cudaError_t e = fused_dispatch(C, set, false);
    return e != cudaSuccess ? e : fused_dispatch(C, set, true);
}

// Rows per group G, ring depth NB and the grid: over G in {1, 2, 4, 8, 16}
// and NB in {2, 3, 4} whose shared memory fits, the most threads resident
// per SM (blocks per SM from the occupancy calculator), then the most rows
// staged per block (deeper pipeline), then the larger G (fewer barriers per
// row); the grid fills every SM with that many blocks.
bool sv_fused_plan(int Ns, int P, int *G_out, int *NB_out, int *ctas_out) {
    int C, T;
    if (P % 2 || Ns < 1 || !fused_shape(P, &C, &T)) return false;  // rows 16-byte aligned; columns in registers
    int dev = 0, sms = 152, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (prepare_sv_fused(P) != cudaSuccess) return false;
    int best_G = 0, best_NB = 0, best_blocks = 0, best_threads = 0, best_rows = 0;
    for (int G = 1; G <= kFsMaxG; G *= 2)
        for (int NB = 2; NB <= kFsMaxNB; NB++) {
            const size_t smem = fused_smem(C * T, G, NB);
            if (smem > size_t(optin) - 1024) continue;
            int blocks = 0;
            const cudaError_t e = fused_dispatch(C, [&](auto fn) {
                return cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, T, smem);
            });
            if (e != cudaSuccess || blocks < 1) continue;
            const int threads = std::min(blocks * T, 2048), rows = G * NB;
            if (threads > best_threads || (threads == best_threads && (rows > best_rows || (rows == best_rows && G > best_G)))) {
                best_threads = threads;
                best_rows = rows;
                best_G = G;
                best_NB = NB;
                best_blocks = blocks;
            }
        }
    if (!best_G) return false;
    *G_out = best_G;
    *NB_out = best_NB;
    *ctas_out = std::max(1, std::min(sms * best_blocks, (Ns + best_G - 1) / best_G));
    return true;
}

cudaError_t launch_sv_fused(int Ns, int P, int G, int NB, int ctas, const double *O, const double *v, double *ypart,
                            int *err, const int *guard, cudaStream_t st, bool o_split) {
    FusedSvArgs a{Ns, P, G, NB, o_split ? 1 : 0, O, v, ypart, err, guard};
    int C, T;
    if (!fused_shape(P, &C, &T)) return cudaErrorInvalidValue;
    const size_t smem = fused_smem(C * T, G, NB);
    return fused_dispatch(
        C,
        [&](auto fn) {
            fn<<<ctas, T, smem, st>>>(a);
            return cudaGetLastError();
        },
        o_split);
}

}  // namespace nqes
