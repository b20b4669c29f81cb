// S·v over the dense FP64 log-derivatives in ONE read of O, off the FP64 pipe.
//
// The S·v of code/rbm.cc:660-683 over the stored O (real arithmetic, the
// FP64 and certified forms) is y = O^T (O v) plus diagonal and rank-one terms
// that the Lanczos kernels add. Two separate passes (u = O v, then O^T u)
// read the Ns × P matrix twice and run two FP64 FMAs per entry on a part whose
// FP64 pipe retires about two FMAs per SM per clock: 0.41 ms at N32 M64 K2.
//
// Here a persistent CTA per SM owns a contiguous range of rows and streams
// them through shared memory in groups of G rows, double-buffered by bulk
// copies (cp.async.bulk on an mbarrier, bounded waits). For each staged group
//   pass 1: u_r = O_r . v for the group's rows, block-wide, and
//   pass 2: y_p += O_rp u_r into the CTA's partial of O^T u (registers),
// both from shared memory, so O leaves HBM once per S·v. The arithmetic is
// double-float on the FP32 pipe: each FP64 entry d is split exactly-enough
// into hi + lo floats by integer operations (hi = d cut to 24 significant
// bits, lo = the remaining 29 bits rounded to 24: |d - hi - lo| <= 2^-48 |d|),
// products are formed with their FMA error terms, sums are TwoSum-compensated.
// The relative error of u and of the partials against FP64 sums of the same
// terms is a few 2^-48 per term of sum |O v| (about 1e-14 at these sizes),
// inside the 1e-12 parity bound. Entries below 2^-126 in magnitude count as
// zero (absolute error under 1e-38); an entry of magnitude 2^127 or more, or a
// non-finite one, sets kErrNonFinite.
//
// Each CTA writes its partial y (converted to FP64) to ypart[cta]; the
// Lanczos epilogue sums the partials over CTAs in a fixed order, so results
// do not depend on timing.
#include <algorithm>

#include "nqes_internal.h"
#include "tma_stage.cuh"

namespace nqes {
namespace {

constexpr int kFsThreads = 512;  // 16 warps
constexpr int kFsWarps = kFsThreads / 32;
constexpr int kFsMaxG = 8;       // rows per staged group (registers per thread: 2 per row)

// hi + lo = d to 2^-48 relative (see the file comment); returns false when
// |d| >= 2^127 or d is not finite.
__device__ __forceinline__ bool split_d(double d, float &hi, float &lo) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
    const unsigned hw = unsigned(b >> 32), lw = unsigned(b);
    const unsigned ax = hw & 0x7fffffffu, sgn = hw & 0x80000000u;
    // biased exponent e = ax >> 20; hi is representable as a normal float for
    // 897 <= e <= 1150: exponent e - 896, mantissa the top 23 of d's 52 bits
    const bool nrm = ax >= 0x38100000u;
    const unsigned hb = __funnelshift_l(lw, ax - 0x38000000u, 3);
    hi = __uint_as_float(nrm ? (hb | sgn) : sgn);
    // lo = sign * r * 2^(e - 1075) with r the low 29 mantissa bits; the scale
    // is a normal float for e >= 949 (below, |lo| < 2^-149 |...|: dropped)
    const unsigned e = ax >> 20;
    const float sc = __uint_as_float((e - 948u) << 23);
    const float l = __uint2float_rn(lw & 0x1fffffffu) * sc;
    lo = e >= 949u ? __uint_as_float(__float_as_uint(l) | sgn) : 0.f;
    return ax < 0x47f00000u;
}

// (sh, sl) += (ah + al) (bh + bl): the product to 2^-48 relative (its FMA
// error term and the two cross terms), added with TwoSum into sh and the
// rounding error and low terms into sl.
__device__ __forceinline__ void df_mac(float &sh, float &sl, float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    float e = __fmaf_rn(ah, bh, -p);
    e = __fmaf_rn(ah, bl, e);
    e = __fmaf_rn(al, bh, e);
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// (ah, al) += (bh, bl)
__device__ __forceinline__ void df_add(float &ah, float &al, float bh, float bl) {
    const float s = __fadd_rn(ah, bh);
    const float bb = __fsub_rn(s, ah);
    const float err = __fadd_rn(__fsub_rn(ah, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    ah = s;
    al = __fadd_rn(al, __fadd_rn(err, bl));
}

__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

struct FusedSvArgs {
    int Ns, P, G;
    const double *O, *v;
    double *ypart;  // gridDim.x × P
    int *err;
    const int *guard;
};

// Block: kFsThreads threads; thread t owns columns p = t + c kFsThreads
// (c < C), holding v's split and its partial of O^T u for them in registers.
template <int C>
__global__ void __launch_bounds__(kFsThreads, 1) k_sv_fused(FusedSvArgs a) {
    extern __shared__ __align__(16) unsigned char fs_smem[];
    if (loop_guard_off(a.guard)) return;
    const int P = a.P, G = a.G, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    double *buf0 = reinterpret_cast<double *>(fs_smem);
    double *buf1 = buf0 + size_t(G) * P;
    float2 *red = reinterpret_cast<float2 *>(buf1 + size_t(G) * P);  // [kFsWarps][G]
    float2 *us = red + kFsWarps * G;                                  // [G]
    uint64_t *mbar = reinterpret_cast<uint64_t *>(us + kFsMaxG);      // [2] (8-byte aligned: G, P even or 8-byte sized)
    const int r0 = int(int64_t(a.Ns) * blockIdx.x / gridDim.x), r1 = int(int64_t(a.Ns) * (blockIdx.x + 1) / gridDim.x);
    const int ngroups = (r1 - r0 + G - 1) / G;

    float vh[C], vl[C], yh[C], yl[C];
    bool range_ok = true;
#pragma unroll
    for (int c = 0; c < C; c++) {
        const int p = tid + c * kFsThreads;
        vh[c] = vl[c] = yh[c] = yl[c] = 0.f;
        if (p < P) range_ok &= split_d(a.v[p], vh[c], vl[c]);
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
        // pass 1: split the staged entries in place (each thread its own
        // columns, read back only by itself) and form the rows' dot products
        float sh[kFsMaxG], sl[kFsMaxG];
#pragma unroll
        for (int r = 0; r < kFsMaxG; r++) sh[r] = sl[r] = 0.f;
#pragma unroll
        for (int c = 0; c < C; c++) {
            const int p = tid + c * kFsThreads;
            if (p < P) {
#pragma unroll
                for (int r = 0; r < kFsMaxG; r++) {
                    if (r < nr) {
                        double *at = buf + size_t(r) * P + p;
                        float oh, ol;
                        range_ok &= split_d(*at, oh, ol);
                        *reinterpret_cast<float2 *>(at) = make_float2(oh, ol);
                        df_mac(sh[r], sl[r], oh, ol, vh[c], vl[c]);
                    }
                }
            }
        }
        // block sums of the rows: warp shuffles, then the warps in order
#pragma unroll
        for (int r = 0; r < kFsMaxG; r++) {
            if (r < nr) {
                float h = sh[r], l = sl[r];
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const float oh = __shfl_down_sync(0xffffffffu, h, off), ol = __shfl_down_sync(0xffffffffu, l, off);
                    df_add(h, l, oh, ol);
                }
                if (lane == 0) red[warp * G + r] = make_float2(h, l);
            }
        }
        __syncthreads();
        if (tid < nr) {
            float h = 0.f, l = 0.f;
            for (int w = 0; w < kFsWarps; w++) df_add(h, l, red[w * G + tid].x, red[w * G + tid].y);
            us[tid] = make_float2(h, l);
        }
        __syncthreads();
        // pass 2: y_p += O_rp u_r over the group's rows
#pragma unroll
        for (int r = 0; r < kFsMaxG; r++) {
            if (r < nr) {
                const float2 u = us[r];
#pragma unroll
                for (int c = 0; c < C; c++) {
                    const int p = tid + c * kFsThreads;
                    if (p < P) {
                        const float2 o = *reinterpret_cast<const float2 *>(buf + size_t(r) * P + p);
                        df_mac(yh[c], yl[c], o.x, o.y, u.x, u.y);
                    }
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
        const int p = tid + c * kFsThreads;
        if (p < P) a.ypart[size_t(blockIdx.x) * P + p] = double(yh[c]) + double(yl[c]);
    }
}

template <int C> const void *fused_fn() { return reinterpret_cast<const void *>(k_sv_fused<C>); }

int fused_cols(int P) {
    const int c = (P + kFsThreads - 1) / kFsThreads;
    return c <= 1 ? 1 : c <= 2 ? 2 : c <= 4 ? 4 : c <= 8 ? 8 : c <= 12 ? 12 : 16;
}

size_t fused_smem(int P, int G) {
    return size_t(2) * G * P * sizeof(double) + (size_t(kFsWarps) * G + kFsMaxG) * sizeof(float2) + 2 * sizeof(uint64_t);
}

}  // namespace

bool sv_fused_plan(int Ns, int P, int *G_out, int *ctas_out) {
    if (P % 2 || P > 16 * kFsThreads || Ns < 1) return false;  // rows 16-byte aligned; columns in registers
    int dev = 0, sms = 152, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    int G = kFsMaxG;
    while (G > 1 && fused_smem(P, G) > size_t(optin) - 1024) G--;
    if (fused_smem(P, G) > size_t(optin) - 1024) return false;
    *G_out = G;
    *ctas_out = std::max(1, std::min(sms, (Ns + G - 1) / G));
    return true;
}

cudaError_t prepare_sv_fused(int P) {
    switch (fused_cols(P)) {
    case 1: return allow_max_dynamic_smem(fused_fn<1>());
    case 2: return allow_max_dynamic_smem(fused_fn<2>());
    case 4: return allow_max_dynamic_smem(fused_fn<4>());
    case 8: return allow_max_dynamic_smem(fused_fn<8>());
    case 12: return allow_max_dynamic_smem(fused_fn<12>());
    default: return allow_max_dynamic_smem(fused_fn<16>());
    }
}

cudaError_t launch_sv_fused(int Ns, int P, int G, int ctas, const double *O, const double *v, double *ypart, int *err,
                            const int *guard, cudaStream_t st) {
    FusedSvArgs a{Ns, P, G, O, v, ypart, err, guard};
    const size_t smem = fused_smem(P, G);
    switch (fused_cols(P)) {
    case 1: k_sv_fused<1><<<ctas, kFsThreads, smem, st>>>(a); break;
    case 2: k_sv_fused<2><<<ctas, kFsThreads, smem, st>>>(a); break;
    case 4: k_sv_fused<4><<<ctas, kFsThreads, smem, st>>>(a); break;
    case 8: k_sv_fused<8><<<ctas, kFsThreads, smem, st>>>(a); break;
    case 12: k_sv_fused<12><<<ctas, kFsThreads, smem, st>>>(a); break;
    default: k_sv_fused<16><<<ctas, kFsThreads, smem, st>>>(a); break;
    }
    return cudaGetLastError();
}

}  // namespace nqes
