// Mixed-precision sampler, decision-warp form (real weights, up to 32 hidden
// units per lane). Same chains and same certified FP32 decisions as the
// block form in kernels_sample_mixed.cu (code/rbm.cc:530-552 trajectories),
// laid out for latency:
//
// One warp (warp 0 of the chain's CTA) runs every proposal of a row. Its
// lanes form K groups of G lanes (G the largest power of two <= 32/K); lane
// (kk, jl) owns hidden units j = jl*U .. jl*U+U-1 of RBM kk and keeps their
// tanh(theta) in registers for the whole row. A proposal is U fused
// multiply-adds, a log2(G)-level shuffle tree inside each group and K
// broadcasts; every lane then holds all K products and takes the accept
// decision itself, so a proposal needs no CTA barrier and no shared-memory
// round trip. An accepted flip updates tanh by the exact identity
// t' = (t c - sigma s) / f with f already at hand: no FP64 instruction on the
// proposal path.
//
// At the end of a row that changed, the whole CTA (the other warps wait at a
// barrier meanwhile) rebuilds that row's theta from the spins as double-float
// sums of b and the +-w, recomputes tanh with tanhf, and recomputes the row of
// Phi in FP64, so every row of Phi is exact (to ~1e-12 relative) whenever
// another row is swept: a decision's bound only carries the drift of the
// swept row. The error model of a proposal is stated at run_row. A decision
// the bound cannot make, or any value out of FP32's normal range, goes to the
// exact path: the swept row's current and proposed entries in FP64 from theta
// and the reference's test u |det Phi|^2 <= |det Phi'|^2 in FP64.
//
// The step's tables (cosh 2w, sinh 2w, w as hi + lo; padded to MP units per
// row so that padding factors are exactly 1) are bulk-copied into shared
// memory (cp.async.bulk on an mbarrier) when the launch plan allows.
#pragma once
#include <algorithm>
#include <cfloat>

#include "nqes_internal.h"
#include "pcg64.cuh"
#include "tma_stage.cuh"

namespace nqes {

namespace {

constexpr float kU = 5.9604645e-8f;  // FP32 unit roundoff 2^-24
constexpr int kMaxSpinWords = 8;

// Register cap of the decision-warp kernel below 16 units per lane.
#ifndef NQES_DW_MAXNREG
#define NQES_DW_MAXNREG 128
#endif

__device__ __forceinline__ bool down_bit(const uint64_t *s, int i) { return (s[i >> 6] >> (i & 63)) & 1ULL; }
__device__ __forceinline__ int expo32(float x) {
    const int b = (__float_as_int(x) >> 23) & 0xff;
    return b == 0 ? 0 : b - 127;
}

// (ah, al) += (bh, bl): double-float addition from two-sum (Knuth) and a
// final fast two-sum; relative error a few 2^-48 of max(|a|, |b|).
__device__ __forceinline__ void df_add(float &ah, float &al, float bh, float bl) {
    const float s = ah + bh;
    const float bb = s - ah;
    float e = (ah - (s - bb)) + (bh - bb);
    e += al + bl;
    const float h = s + e;
    al = e - (h - s);
    ah = h;
}

struct DSmem {
    double *phi, *pinv, *Dm, *jk, *lsum, *jpart;
    float *th_hi, *th_lo, *t, *rat, *bsig, *Bm;
    uint64_t *spin, *spin_snap, *mbar;
    int *flag;
    double *t64;  // FP64 outputs: tanh of the exact theta [K*K][MP]
    float *tabs;  // staged tables (cosh 2w, sinh 2w, w hi, w lo), 4 * K*N*MP floats
    // the tables the kernel reads: staged copies or global memory
    const float *tc, *ts, *twh, *twl;
};

// One table of K*N*MP floats in bytes (a multiple of 16: MP*4 >= 32).
__host__ __device__ inline size_t dw_table_bytes(int N, int MP, int K) { return size_t(K) * N * MP * 4; }

__host__ __device__ inline size_t dsmem_bytes(int N, int MP, int K, bool staged, bool out64 = false) {
    const size_t KK = size_t(K) * K;
    const size_t nd = 3 * KK + 4 + 32 + 32 * 4;
    const size_t nf = 3 * KK * MP + 2 * KK * N + KK;
    size_t base = nd * 8 + 16 + ((nf * 4 + 15) / 16) * 16 + 16 * kMaxSpinWords + 8 + 4 * 4;  // 16: alignment pad
    if (out64) base += 16 + KK * MP * 8;
    return staged ? base + 16 + 4 * dw_table_bytes(N, MP, K) : base;
}

__device__ inline DSmem dcarve(unsigned char *base, int N, int MP, int K, bool out64) {
    const int KK = K * K;
    DSmem s;
    double *d = reinterpret_cast<double *>(base);
    s.phi = d; d += KK;
    s.pinv = d; d += KK;
    s.Dm = d; d += KK;
    s.jk = d; d += 4;
    s.lsum = d; d += 32;
    s.jpart = d; d += 32 * 4;
    // float arrays start on a 16-byte boundary (vector loads of theta and tanh)
    unsigned char *fb = reinterpret_cast<unsigned char *>(d);
    fb += (16 - (reinterpret_cast<uintptr_t>(fb) & 15)) & 15;
    float *f = reinterpret_cast<float *>(fb);
    s.th_hi = f; f += KK * MP;
    s.th_lo = f; f += KK * MP;
    s.t = f; f += KK * MP;
    s.rat = f; f += KK * N;
    s.bsig = f; f += KK * N;
    s.Bm = f; f += KK;
    unsigned char *p = reinterpret_cast<unsigned char *>(f);
    p += (8 - (reinterpret_cast<uintptr_t>(p) & 7)) & 7;
    s.spin = reinterpret_cast<uint64_t *>(p);
    s.spin_snap = s.spin + kMaxSpinWords;
    s.mbar = s.spin_snap + kMaxSpinWords;
    s.flag = reinterpret_cast<int *>(s.mbar + 1);
    unsigned char *tb = reinterpret_cast<unsigned char *>(s.flag + 4);
    tb += (16 - (reinterpret_cast<uintptr_t>(tb) & 15)) & 15;
    s.t64 = reinterpret_cast<double *>(tb);
    if (out64) {
        tb += size_t(KK) * MP * 8;
        tb += (16 - (reinterpret_cast<uintptr_t>(tb) & 15)) & 15;
    }
    s.tabs = reinterpret_cast<float *>(tb);
    return s;
}

// Cofactor of (r, c) and the sum of |Leibniz terms| of that minor, K <= 4.
__device__ void cofactor_abs(const double *m, int K, int r, int c, double &cof, double &cabs) {
    if (K == 1) {
        cof = 1.0;
        cabs = 1.0;
        return;
    }
    double sub[9], sab[9];
    int t = 0;
    for (int a = 0; a < K; a++) {
        if (a == r) continue;
        for (int b = 0; b < K; b++)
            if (b != c) {
                sub[t] = m[a * K + b];
                sab[t] = fabs(m[a * K + b]);
                t++;
            }
    }
    const double d = small_det(sub, K - 1);
    double p;
    if (K == 2) {
        p = sab[0];
    } else if (K == 3) {
        p = sab[0] * sab[3] + sab[1] * sab[2];
    } else {
        p = sab[0] * (sab[4] * sab[8] + sab[5] * sab[7]) + sab[1] * (sab[3] * sab[8] + sab[5] * sab[6]) +
            sab[2] * (sab[3] * sab[7] + sab[4] * sab[6]);
    }
    cof = ((r + c) & 1) ? -d : d;
    cabs = p;
}

// Row k from the spins: theta (double-float sums of b and +-w), tanh(theta)
// in FP32, and Phi[k][.] in FP64, scaled by a power of two that brings the
// row's largest entry near 1:
//   Phi[k][kk] ~ P_kk exp(A_kk - max A),  A_kk = sum_i sigma_i a_i + sum_j |theta_j|,
//   P_kk = prod_j (1 + e^{-2|theta_j|})  (each factor in (1, 2]),
// e^{-2|theta|} per hidden unit from the exp table (exp_neg_tab) and one exp
// per entry. Block-wide; ends with a barrier.
__device__ void rebuild_row(const MixedArgs &A, DSmem &sm, int k) {
    const int N = A.sh.N, M = A.sh.M, K = A.sh.K, NW = A.sh.NW, MP = A.MP;
    const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = T >> 5;
    const uint64_t *sk = sm.spin + k * NW;
    // four adjacent hidden units per thread (MP is a multiple of 8): one float4
    // of each table per spin and four independent double-float chains, so a
    // thread has four loads and sums in flight instead of one
    for (int qd = tid; qd < K * MP / 4; qd += T) {
        const int kk = int(fdiv(unsigned(qd * 4), A.fdMP)), j0 = qd * 4 - kk * MP, q = k * K + kk;
        const float4 bh4 = *reinterpret_cast<const float4 *>(A.bh + kk * MP + j0);
        const float4 bl4 = *reinterpret_cast<const float4 *>(A.bl + kk * MP + j0);
        float h[4] = {bh4.x, bh4.y, bh4.z, bh4.w}, l[4] = {bl4.x, bl4.y, bl4.z, bl4.w};
#pragma unroll 2
        for (int i = 0; i < N; i++) {
            const size_t o = (size_t(kk) * N + i) * MP + j0;
            const float4 wh = *reinterpret_cast<const float4 *>(sm.twh + o);
            const float4 wl = *reinterpret_cast<const float4 *>(sm.twl + o);
            const bool dn = down_bit(sk, i);
            df_add(h[0], l[0], dn ? -wh.x : wh.x, dn ? -wl.x : wl.x);
            df_add(h[1], l[1], dn ? -wh.y : wh.y, dn ? -wl.y : wl.y);
            df_add(h[2], l[2], dn ? -wh.z : wh.z, dn ? -wl.z : wl.z);
            df_add(h[3], l[3], dn ? -wh.w : wh.w, dn ? -wl.w : wl.w);
        }
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int j = j0 + e;
            const bool in = j < M;
            sm.th_hi[q * MP + j] = in ? h[e] : 0.f;
            sm.th_lo[q * MP + j] = in ? l[e] : 0.f;
            sm.t[q * MP + j] = in ? tanhf(h[e]) : 0.f;
        }
    }
    __syncthreads();
    // sums of A and products P over slots (kk, part), max(1, 4 / K) parts per
    // RBM, each a strided share of the row's hidden units summed by one warp
    // (lanes, then the warp's fixed tree), the slots taken by the warps in
    // turn: the same order, and so the same Phi, for any warps per chain
    const int wpk = max(1, 4 / K);
    for (int v = warp; v < K * wpk; v += nwarp) {
        const int kk = v / wpk, part = v - kk * wpk, q = k * K + kk;
        double lin = 0.0, pr = 1.0;
        for (int j = lane + 32 * part; j < M; j += 32 * wpk) {
            const double th = double(sm.th_hi[q * MP + j]) + double(sm.th_lo[q * MP + j]);
            lin += fabs(th);
            pr *= 1.0 + exp_neg_tab(2.0 * fabs(th), A.etab);
        }
        if (part == 0)
            for (int i = lane; i < N; i += 32) lin += down_bit(sk, i) ? -A.a64[kk * N + i] : A.a64[kk * N + i];
        lin = warp_sum(lin);
        pr = warp_prod(pr);
        if (lane == 0) {
            sm.jpart[2 * v] = lin;
            sm.jpart[2 * v + 1] = pr;
        }
    }
    __syncthreads();
    if (warp == 0) {
        // lanes kk < K: the entry from its slots; then the row's scaling
        double a = -1e308, pp = 0.0;
        if (lane < K) {
            a = 0.0;
            pp = 1.0;
            for (int part = 0; part < wpk; part++) {
                a += sm.jpart[2 * (lane * wpk + part)];
                pp *= sm.jpart[2 * (lane * wpk + part) + 1];
            }
        }
        double mx = a;
        for (int o = 1; o < 4; o <<= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mx = __shfl_sync(0xffffffffu, mx, 0);
        // e^{a - mx} from the table (a dozen FP64 instructions instead of the
        // library exp's few dozen, each a full warp's turn on the FP64 pipe);
        // exp itself only where an entry lies more than e^-40 below the largest
        const double x = lane < K ? mx - a : 0.0;
        const double e = lane < K ? pp * (x < 40.0 ? exp_neg_tab(x, A.etab) : exp(-x)) : 0.0;
        int ex = lane < K ? expo(e) : -100000;
        for (int o = 1; o < 4; o <<= 1) ex = max(ex, __shfl_xor_sync(0xffffffffu, ex, o));
        ex = __shfl_sync(0xffffffffu, ex, 0);
        if (lane < K) sm.phi[k * K + lane] = scale2(e, -ex);
    }
    __syncthreads();
}

// All proposals of row k, run by one warp. Returns whether the row changed.
//
// Error model of the FP32 proposal (u = 2^-24).
//
// tanh. tanh(theta) of the lane's units is held in FP32 with an absolute
// error of at most Et (one bound per RBM, the same in every lane): 5u after
// the row's rebuild (tanhf). An accepted flip updates t' = (t c - sigma s) / f,
// a map with derivative 1/f^2, and rounds with eps <= u (2 max_j cond_j + 5),
// cond_j = (c + |s|)/(c - |s|) >= (|c| + |t s|)/|f| (|t| <= 1). Two bounds hold
// and the smaller is kept:
//  - stepwise: Et' = Et max_j 1/f_j^2 + eps, with 1/f^2 <= 1/(c - |s|)^2;
//  - telescoped: 1/f_j = cosh(theta_j) / cosh(theta_j'), so the product of the
//    derivatives from any step to now is cosh^2(theta_then) / cosh^2(theta_now)
//    <= cosh^2(|theta_0| + 2 sum_i |w_ij|) =: Am (each spin of the row flips at
//    most once per row). Evaluating the derivative between the held and the
//    exact t adds a factor (1 - Et q)^-2 <= 1 + 2.05 Et q per step (Et q <=
//    0.01), q = max_j |s|/(c - |s|) = (max_j cond_j - 1) / 2. Hence
//    Et <= Am F (5u + sum of eps), F the product of those factors.
// A factor f_j = c - sigma t s then has relative error at most u (cond_j + 1) +
// Et |s| / (c - |s|), and the product over the row's M factors (M - 1 + 16
// roundings, the 16 also covering the FP64 tables' own rounding)
//   beta = u (sum_j cond_j + 2M + 16) + Et sum_j |s_j| / (c_j - |s_j|).
// The per-(kk, i) sums and maxima come from a table built with the weights.
//
// Decision. The FP64 test u |det|^2 <= |det'|^2 is u <= |rho|^2 with rho =
// det'/det = sum_kk re_kk g_kk / sum_kk g_kk (g_kk = Phi[k][kk] cof_kk; re_kk
// the entry's ratio, including e^{-2 sigma a}). The held g_kk differ from the
// exact ones by at most dr |g_kk| + ga_kk (dr: the row's relative drift from
// accepted FP32 flips; ga: the FP64 rows' own error) and the held det from
// sum_kk g_kk by at most edet. The drift enters only through
// sum_kk (re_kk - rho) (g_kk - g*_kk) / det, which is small when the states
// are alike, so with rh = s / det the error of rh is at most
//   E = [sum_kk |g| |re| (beta + 3u) + 1.03 sum_kk (dr |g| + ga) (|re - rh| + 1.02 bmax |re|)
//        + (K + 1) u sum_kk |x| + |rh| edet] / |det| (1 + 2q) + 3u |rh|,
//   q = (1.03 dr sum|g| + sum ga + edet) / |det|  (required < 1/2, so that
//   1 / (1 - q) <= 1 + 2q).
// A decision the margins (16u on each side) cannot make goes to the exact
// path.
template <int K, int U>
__device__ bool run_row(const MixedArgs &A, DSmem &sm, int k, Pcg64 &rng, unsigned long long &nacc,
                        unsigned long long &nexact) {
    constexpr int G = K == 1 ? 32 : (K == 2 ? 16 : 8);
    const int N = A.sh.N, M = A.sh.M, NW = A.sh.NW, MP = A.MP;
    const int lane = threadIdx.x & 31;
    const int gkk = lane / G, gjl = lane % G;
    const bool active = gkk < K;
    const int kkl = active ? gkk : 0;  // idle lanes (K = 3) read RBM 0's tables and contribute factor 1
    const int q = k * K + kkl, base = gjl * U;

    float t[U];
#pragma unroll
    for (int u = 0; u < U; u++) t[u] = sm.t[q * MP + base + u];
    bool live[U];  // unit inside the RBM (not padding) and lane in a group
#pragma unroll
    for (int u = 0; u < U; u++) live[u] = active && base + u < M;
    uint64_t sk0 = sm.spin[k * NW], sk1 = NW > 1 ? sm.spin[k * NW + 1] : 0ULL;
    auto bit = [&](int b) -> bool { return ((b < 64 ? sk0 : sk1) >> (b & 63)) & 1ULL; };

    // Decision state, identical in every lane: exact cofactors of row k (the
    // other rows are exact), the row's entries, g, det and 1/det with the
    // error bounds of the model above.
    double cofd[K], cabsd[K];
    float phik[K], g[K], ga[K], Et[K], Eacc[K], Fq[K], Am[K], Qs[K];
    // third tanh bound for the wider shapes: the amplification from step s to
    // now is at most cosh^2 theta_s = 1 / (1 - T_s^2) <= 1 / (1 - M_s^2), M_s the
    // RBM's largest |tanh| after step s (plus its error), so E_t <= F Qs with
    // Qs = sum_s eps_s / (1 - M_s^2); one group max per accepted flip
    constexpr bool kTmax = U * K >= 16;
    float det32, rdet, edet, gsum, gasum, dr;
    auto exact_state = [&](const double *pp, double det) {
        double perm = 0.0;
        gsum = 0.f;
        gasum = 0.f;
#pragma unroll
        for (int kk = 0; kk < K; kk++) {
            const double p = pp[kk];
            phik[kk] = float(p);
            g[kk] = float(p * cofd[kk]);
            ga[kk] = float(fabs(p) * cabsd[kk] * 0x1p-30);  // rows exact to far better than 2^-30
            perm += fabs(p) * cabsd[kk];
            gsum += fabsf(g[kk]);
            gasum += ga[kk];
        }
        det32 = float(det);
        rdet = __frcp_rn(det32);  // correctly rounded, as the bound assumes
        edet = kU * (fabsf(det32) + gsum) * 1.01f + float(perm * 0x1p-50);
        dr = 2.f * kU;
    };
    {
        double det = 0.0, pp[K];
#pragma unroll
        for (int kk = 0; kk < K; kk++) {
            cofactor_abs(sm.phi, K, k, kk, cofd[kk], cabsd[kk]);
            pp[kk] = sm.phi[k * K + kk];
            det += pp[kk] * cofd[kk];
            Et[kk] = 5.f * kU;
            Eacc[kk] = 5.f * kU;
            Fq[kk] = 1.f;
        }
        exact_state(pp, det);
        // Am = cosh^2(|theta_0| + 2 max_j sum_i |w_ij|), |theta_0| = atanh(max |t|)
        float tm = 0.f;
#pragma unroll
        for (int u = 0; u < U; u++)
            if (live[u]) tm = fmaxf(tm, fabsf(t[u]));
#pragma unroll
        for (int o = G >> 1; o > 0; o >>= 1) tm = fmaxf(tm, __shfl_xor_sync(0xffffffffu, tm, o));
#pragma unroll
        for (int kk = 0; kk < K; kk++) {
            const float tk = __shfl_sync(0xffffffffu, tm, kk * G) + 6.f * kU;
            const float ch = coshf(fmaf(atanhf(tk), 1.f + 8.f * kU, __ldg(A.bnd + 4 * K * N + kk)));
            Am[kk] = tk < 0.9999f ? ch * ch * (1.f + 1e-5f) : INFINITY;
            Qs[kk] = tk < 0.9999f ? 5.f * kU * (1.f + 16.f * kU) * __frcp_ru((1.f - tk) * (1.f + tk)) : INFINITY;
        }
    }
    bool changed = false;

    for (int i = 0; i < N; i++) {
        const bool down = bit(i);
        const size_t row = (size_t(kkl) * N + i) * MP + base;
        float cq[U], sq[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            cq[u] = sm.tc[row + u];
            sq[u] = sm.ts[row + u];
        }
        float ea[K];
        float4 bd[K];
#pragma unroll
        for (int kk = 0; kk < K; kk++) {
            ea[kk] = __ldg((down ? A.edn : A.eup) + kk * N + i);
            bd[kk] = __ldg(reinterpret_cast<const float4 *>(A.bnd) + kk * N + i);
        }
        const uint64_t draw = pcg_next(rng);
        const float u32 = __ull2float_rn(draw) * 0x1p-64f;

        // factors f = c - sigma t s and their product within the lane's group,
        // as up to four interleaved partial products (a shorter dependent chain;
        // the same number of roundings, so beta still bounds it)
        constexpr int NPP = U < 4 ? U : 4;
        float f[U], pp[NPP];
#pragma unroll
        for (int e = 0; e < NPP; e++) pp[e] = 1.f;
#pragma unroll
        for (int u = 0; u < U; u++) {
            f[u] = fmaf(down ? t[u] : -t[u], sq[u], cq[u]);
            if (live[u]) pp[u % NPP] *= f[u];
        }
        float prod = pp[0];
#pragma unroll
        for (int e = 1; e < NPP; e++) prod *= pp[e];
#pragma unroll
        for (int o = G >> 1; o > 0; o >>= 1) prod *= __shfl_xor_sync(0xffffffffu, prod, o);
        float x[K], re[K], beta[K], s = 0.f, sax = 0.f, bmax = 0.f;
#pragma unroll
        for (int kk = 0; kk < K; kk++) {
            const float rr = __shfl_sync(0xffffffffu, prod, kk * G);
            beta[kk] = fmaf(Et[kk], bd[kk].y, bd[kk].x);
            re[kk] = rr * ea[kk];
            x[kk] = re[kk] * g[kk];
            s += x[kk];
            sax += fabsf(x[kk]);
            bmax = fmaxf(bmax, beta[kk]);
        }
        const float rh = s * rdet;
        float e1 = 0.f, e2 = 0.f;
#pragma unroll
        for (int kk = 0; kk < K; kk++) {
            const float ar = fabsf(re[kk]), ag = fabsf(g[kk]);
            e1 = fmaf(ag * ar, beta[kk] + 3.f * kU, e1);
            e2 = fmaf(fmaf(dr, ag, ga[kk]), fmaf(1.02f * bmax, ar, fabsf(re[kk] - rh)), e2);
        }

        bool acc = false, exact_path = false;
        {
            const float ad = fabsf(det32), ard = fabsf(rdet), arh = fabsf(rh);
            const float q = fmaf(1.03f * dr, gsum, gasum + edet) * ard;
            const float num = fmaf(1.03f, e2, e1) + fmaf(float(K + 1) * kU, sax, arh * edet);
            // 1 / (1 - q) <= 1 + 2q for q <= 1/2 (required below): no division
            const float E = fmaf(1.02f * num * ard, fmaf(2.f, q, 1.f), 3.f * kU * arh);
            const float lo = arh - E, hi = arh + E;
            if (A.exact_all || !(ad > 1e-15f) || !(ad < 1e15f) || !(bmax < 0.01f) || !(q < 0.5f))
                exact_path = true;  // det == 0 (accepted, code/rbm.cc:542), range, loose bound
            else if (lo > 0.f && lo * lo * (1.f - 16.f * kU) >= u32 * (1.f + 16.f * kU))
                acc = true;
            else if (!(hi * hi * (1.f + 16.f * kU) < u32 * (1.f - 16.f * kU)))
                exact_path = true;  // NaN lands here as well
        }
        if (exact_path) {
            // Row k current and proposed, in FP64. theta of the lane's units is
            // the row's start value (double-float, left in shared memory by the
            // last rebuild of this row) plus 2 sigma w for each spin flipped
            // since (a spin flips at most once per row), four units at a time;
            // then the log cosh sums.
            double lin = 0.0, pr = 1.0, lin2 = 0.0, pr2 = 1.0;
            const uint64_t fl0 = sk0 ^ sm.spin[k * NW], fl1 = NW > 1 ? (sk1 ^ sm.spin[k * NW + 1]) : 0ULL;
            constexpr int UC = U < 4 ? U : 4;
#pragma unroll 1
            for (int u0 = 0; u0 < U; u0 += UC) {
                float h[UC], l[UC];
#pragma unroll
                for (int e = 0; e < UC; e++) {
                    h[e] = sm.th_hi[q * MP + base + u0 + e];
                    l[e] = sm.th_lo[q * MP + base + u0 + e];
                }
#pragma unroll 1
                for (int half = 0; half < 2; half++) {
                    uint64_t f = half ? fl1 : fl0;
                    while (f) {
                        const int i2 = __ffsll(static_cast<long long>(f)) - 1 + 64 * half;
                        f &= f - 1;
                        const size_t o = (size_t(kkl) * N + i2) * MP + base + u0;
                        const float sg = bit(i2) ? -2.f : 2.f;  // sigma now - sigma at the row start
                        float wh[UC], wl[UC];
                        if constexpr (UC == 4) {
                            const float4 a4 = *reinterpret_cast<const float4 *>(sm.twh + o);
                            const float4 b4 = *reinterpret_cast<const float4 *>(sm.twl + o);
                            wh[0] = a4.x; wh[1] = a4.y; wh[2] = a4.z; wh[3] = a4.w;
                            wl[0] = b4.x; wl[1] = b4.y; wl[2] = b4.z; wl[3] = b4.w;
                        } else {
#pragma unroll
                            for (int e = 0; e < UC; e++) {
                                wh[e] = sm.twh[o + e];
                                wl[e] = sm.twl[o + e];
                            }
                        }
#pragma unroll
                        for (int e = 0; e < UC; e++) df_add(h[e], l[e], sg * wh[e], sg * wl[e]);
                    }
                }
#pragma unroll
                for (int e = 0; e < UC; e++) {
                    const int j = base + u0 + e;
                    if (active && j < M) {
                        const double tt = double(h[e]) + double(l[e]);
                        const double w = A.w64[(size_t(kkl) * N + i) * M + j];
                        const double t2 = down ? tt + 2.0 * w : tt - 2.0 * w;
                        lin += fabs(tt);
                        pr *= 1.0 + exp_neg_tab(2.0 * fabs(tt), A.etab);
                        lin2 += fabs(t2);
                        pr2 *= 1.0 + exp_neg_tab(2.0 * fabs(t2), A.etab);
                    }
                }
            }
#pragma unroll
            for (int o = G >> 1; o > 0; o >>= 1) {
                lin += __shfl_xor_sync(0xffffffffu, lin, o);
                lin2 += __shfl_xor_sync(0xffffffffu, lin2, o);
                pr *= __shfl_xor_sync(0xffffffffu, pr, o);
                pr2 *= __shfl_xor_sync(0xffffffffu, pr2, o);
            }
            // A = sum sigma a + sum |theta| and P = prod (1 + e^{-2|theta|}) per RBM,
            // current (c) and proposed (n); entries P exp(A - max A_c), one exp
            // per lane (lanes kk and K + kk)
            double as[K];
#pragma unroll
            for (int kk = 0; kk < K; kk++) {
                as[kk] = 0.0;
                for (int i2 = lane; i2 < N; i2 += 32) {
                    const double ai = A.a64[kk * N + i2];
                    as[kk] += bit(i2) ? -ai : ai;
                }
            }
            double Ac[K], An[K], Pc[K], Pn[K], mx = -1e308;
#pragma unroll
            for (int kk = 0; kk < K; kk++) {
                as[kk] = warp_sum(as[kk]);
                const double ai = A.a64[kk * N + i];
                Ac[kk] = as[kk] + __shfl_sync(0xffffffffu, lin, kk * G);
                An[kk] = as[kk] + (down ? 2.0 * ai : -2.0 * ai) + __shfl_sync(0xffffffffu, lin2, kk * G);
                Pc[kk] = __shfl_sync(0xffffffffu, pr, kk * G);
                Pn[kk] = __shfl_sync(0xffffffffu, pr2, kk * G);
                mx = fmax(mx, Ac[kk]);
            }
            double ev = 0.0;
#pragma unroll
            for (int kk = 0; kk < K; kk++) {
                if (lane == kk) ev = Pc[kk] * exp(Ac[kk] - mx);
                if (lane == K + kk) ev = Pn[kk] * exp(An[kk] - mx);
            }
            // both rows scaled by one power of two that brings the current row's
            // largest entry near 1 (the test is invariant; FP32 copies stay in range)
            double pc[K], pn[K], det_e = 0.0, sx = 0.0;
            int pex = -100000;
#pragma unroll
            for (int kk = 0; kk < K; kk++) {
                pc[kk] = __shfl_sync(0xffffffffu, ev, kk);
                pn[kk] = __shfl_sync(0xffffffffu, ev, K + kk);
                pex = max(pex, expo(pc[kk]));
            }
#pragma unroll
            for (int kk = 0; kk < K; kk++) {
                pc[kk] = scale2(pc[kk], -pex);
                pn[kk] = scale2(pn[kk], -pex);
                det_e += pc[kk] * cofd[kk];
                sx += pn[kk] * cofd[kk];
            }
            acc = det_e == 0.0 || pcg_u01(draw) * (det_e * det_e) <= sx * sx;
            nexact++;
            // continue from the exact row
            exact_state(acc ? pn : pc, acc ? sx : det_e);
        }
        if (acc) {
            // tanh' = (t c - sigma s) / f (code/rbm.cc:185) in FP32, and its bound
#pragma unroll
            for (int u = 0; u < U; u++) t[u] = __fdividef(fmaf(t[u], cq[u], down ? sq[u] : -sq[u]), f[u]);
            float tmx = 0.f;
            if constexpr (kTmax) {
#pragma unroll
                for (int u = 0; u < U; u++)
                    if (live[u]) tmx = fmaxf(tmx, fabsf(t[u]));
#pragma unroll
                for (int o = G >> 1; o > 0; o >>= 1) tmx = fmaxf(tmx, __shfl_xor_sync(0xffffffffu, tmx, o));
            }
#pragma unroll
            for (int kk = 0; kk < K; kk++) {
                Eacc[kk] += bd[kk].w;
                Fq[kk] *= fmaf(1.025f * Et[kk], bd[kk].z - 1.f, 1.f + 2.f * kU);
                const float tel = Am[kk] * Fq[kk] * Eacc[kk] * (1.f + 16.f * kU);
                const float stp = fmaf(Et[kk] * (1.f + 4.f * kU), bd[kk].z, bd[kk].w);
                float e = fminf(tel, stp);
                if constexpr (kTmax) {
                    const float Mk = __shfl_sync(0xffffffffu, tmx, kk * G) + stp + 2.f * kU;
                    Qs[kk] = Mk < 0.9999f ? fmaf(bd[kk].w * (1.f + 16.f * kU), __frcp_ru((1.f - Mk) * (1.f + Mk)), Qs[kk])
                                          : INFINITY;
                    e = fminf(e, Fq[kk] * Qs[kk] * (1.f + 16.f * kU));
                }
                Et[kk] = e;
            }
            if (!exact_path) {
                // row k times r e^{-2 sigma a}: g_kk becomes x_kk (cofactors exclude row k)
                gasum = 0.f;
#pragma unroll
                for (int kk = 0; kk < K; kk++) {
                    phik[kk] *= re[kk];
                    g[kk] = x[kk];
                    ga[kk] *= 1.02f * fabsf(re[kk]);
                    gasum += ga[kk];
                }
                det32 = s;
                rdet = __frcp_rn(s);
                gsum = sax;
                edet = float(K) * kU * sax * 1.01f;
                dr = fmaf(dr, 1.f + bmax + 8.f * kU, fmaf(bmax, 1.01f, 5.f * kU));
            }
            // keep the row's largest entry near 1 (exact power-of-two scaling)
            int ex = -100000;
#pragma unroll
            for (int kk = 0; kk < K; kk++) ex = max(ex, expo32(phik[kk]));
            if (ex > 20 || ex < -20) {
                const float sc = ldexpf(1.f, -ex);
#pragma unroll
                for (int kk = 0; kk < K; kk++) {
                    phik[kk] *= sc;
                    g[kk] *= sc;
                    ga[kk] *= sc;
                }
                det32 *= sc;
                rdet *= ldexpf(1.f, ex);
                edet *= sc;
                gsum *= sc;
                gasum *= sc;
            }
            if (i < 64)
                sk0 ^= 1ULL << i;
            else
                sk1 ^= 1ULL << (i - 64);
            changed = true;
            nacc++;
        }
    }
    if (lane == 0) {
        sm.spin[k * NW] = sk0;
        if (NW > 1) sm.spin[k * NW + 1] = sk1;
    }
    return changed;
}

// One sample (code/rbm.cc:574-657 per sample: local energy and
// log-derivatives) from the chain's current rows of Phi, theta and tanh and the
// configurations `spin`, computed by the threads htid = 0 .. HT - 1 of the
// block, which `sync` synchronises (all of the block's threads, or only the
// helper warps while warp 0 sweeps on).
template <int K, class Sync>
__device__ __forceinline__ void sample_phase(const MixedArgs &A, DSmem &sm, const size_t s, const uint64_t *spin,
                                             const int htid, const int HT, Sync sync) {
    constexpr int KK = K * K;
    const int N = A.sh.N, M = A.sh.M, NW = A.sh.NW, MP = A.MP;
    const int lane = htid & 31, hw = htid >> 5, nhw = HT >> 5;
    const bool writer = htid == 0;
    const bool e64 = A.out64 || A.e64;
    // index math by high multiplies with the launch's divisors (MixedArgs;
    // every index below is far under 2^32 / divisor)
    auto divN = [&](int x) { return int(fdiv(unsigned(x), A.fdN)); };

    // ---- sample: local energy and log-derivatives. Mixed form: FP32 flip
    // ratios combined in FP64, O as its FP32 factors. FP64 outputs: tanh of
    // the exact theta, flip ratios over the FP64 tables, the dense FP64 O row
    // (what the FP64 sampler produces from the same configurations). ----
    if (writer) {
        double pinv[16];
        if (!small_inv(sm.phi, pinv, K)) {
            atomicOr(A.err, kErrSingular);
            for (int t = 0; t < KK; t++) pinv[t] = 0.0;
        }
        for (int t = 0; t < KK; t++) sm.pinv[t] = pinv[t];
    }
    sync();
    {
        // J(s_k) = 2 sum_{i>j} J_ij sigma_i sigma_j (code/rbm.cc:1011-1031): the
        // N x N grid strided over 96 virtual threads (vt takes the pairs
        // vt, vt + 96, ...), partial sums per virtual warp, then the three
        // warps' partials in order. Physical warps take whole virtual warps in
        // turn (the three helper warps one each), so the order, and the
        // result, are the same for any threads.
        for (int vw = hw; vw < 3; vw += nhw) {
            const int vt = vw * 32 + lane;
            double acc[K];
#pragma unroll
            for (int k = 0; k < K; k++) acc[k] = 0.0;
            int i = vt / N, j = vt - (vt / N) * N;
            const int di = 96 / N, dj = 96 - (96 / N) * N;
            while (i < N) {
                if (j < i) {
                    const double p = A.J[size_t(i) * N + j];
#pragma unroll
                    for (int k = 0; k < K; k++) acc[k] += (down_bit(spin + k * NW, i) ^ down_bit(spin + k * NW, j)) ? -p : p;
                }
                j += dj;
                i += di;
                if (j >= N) {
                    j -= N;
                    i++;
                }
            }
#pragma unroll
            for (int k = 0; k < K; k++) {
                acc[k] = warp_sum(acc[k]);
                if (lane == 0) sm.jpart[vw * 4 + k] = acc[k];
            }
        }
        sync();
        if (htid < K) sm.jk[htid] = 2.0 * ((sm.jpart[htid] + sm.jpart[4 + htid]) + sm.jpart[8 + htid]);
    }
    if (e64 && !A.out64) {
        // MIXED: tanh of the exact theta as double-float in the t64 space
        // (layout dfpair_hi per row of MP units): in FP64 (e64 = 1), or
        // (e64 = 2) the row's tanhf(theta_hi) (rebuild_row) plus the
        // first-order term of theta's low part, (1 - t^2) theta_lo, which
        // leaves tanhf's own error (a few 2^-24). Each flip ratio
        // prod_j (c_j + sigma t_j s_j) is a double-float product on the FP32
        // pipe, two units per packed instruction (padded units are exactly
        // 1: t = 0, c = 1, s = 0), to a few 2^-44 per factor.
        for (int e = htid; e < KK * MP; e += HT) {
            const int q = int(fdiv(unsigned(e), A.fdMP)), j = e - q * MP;
            float *tf = reinterpret_cast<float *>(sm.t64) + size_t(q) * 2 * MP + dfpair_hi(j);
            if (A.e64 == 2) {
                const float t = sm.t[e];  // 0 in the padding
                tf[0] = t;
                tf[2] = j < M ? fmaf(-t, t, 1.f) * sm.th_lo[e] : 0.f;
            } else {
                const double tv = j < M ? tanh(double(sm.th_hi[e]) + double(sm.th_lo[e])) : 0.0;
                const float th = float(tv);
                tf[0] = th;
                tf[2] = float(tv - double(th));
            }
        }
        sync();
        double *rat64 = reinterpret_cast<double *>(sm.rat);  // the rat and bsig space: KK*N doubles
        constexpr uint64_t kSign2 = 0x8000000080000000ULL;
        // one row's tables, tanh row and sign
        struct RatRow {
            const float *c, *s, *cl, *sl, *t;
            uint64_t sg;
        };
        auto rat_row = [&](int it) {
            const int q = divN(it), i = it - q * N, k = q / K, kk = q - k * K;
            const bool down = down_bit(spin + k * NW, i);
            const size_t o = (size_t(kk) * N + i) * MP;
            return RatRow{sm.tc + o, sm.ts + o, A.cpl + o, A.spl + o,
                          reinterpret_cast<const float *>(sm.t64) + size_t(q) * 2 * MP,
                          down ? 0ULL : kSign2};  // sigma t = t (spin down) or -t
        };
        // P *= f_j f_j+1 for units j, j + 1 (packed lanes), f = c + sigma t s
        auto rat_step = [&](uint64_t &Ph, uint64_t &Pl, const RatRow &r, int j) {
            const uint64_t ch = *reinterpret_cast<const uint64_t *>(r.c + j);
            const uint64_t sh = *reinterpret_cast<const uint64_t *>(r.s + j);
            const uint64_t cl = __ldg(reinterpret_cast<const unsigned long long *>(r.cl + j));
            const uint64_t sl = __ldg(reinterpret_cast<const unsigned long long *>(r.sl + j));
            const ulonglong2 tt = *reinterpret_cast<const ulonglong2 *>(r.t + 2 * j);
            const uint64_t a = tt.x ^ r.sg, al = tt.y ^ r.sg;
            // f = c + a s as fs + fl (not renormalised): the product a s_hi with its
            // exact error and the cross terms, then ch + p by Fast2Sum, which is exact
            // here because |p| <= |s_hi| <= c_hi (|t| <= 1, sinh 2w < cosh 2w, and
            // rounding keeps the order)
            const uint64_t p = f2_mul(a, sh);
            uint64_t e = f2_fma(a, sh, p ^ kSign2);
            e = f2_fma(a, sl, e);
            e = f2_fma(al, sh, e);
            const uint64_t fs = f2_add(ch, p);
            const uint64_t err = f2_sub(p, f2_sub(fs, ch));
            const uint64_t fl = f2_add(cl, f2_add(err, e));
            // compensated product (Graillat's CompProd, with a double-float
            // factor): Ph *= fs rounded; Pl gathers each product's exact error
            // and the low part's term, scaled along by the later factors
            const uint64_t ph = f2_mul(Ph, fs);
            uint64_t pe = f2_fma(Ph, fs, ph ^ kSign2);
            pe = f2_fma(Ph, fl, pe);
            Pl = f2_fma(Pl, fs, pe);
            Ph = ph;
        };
        // the four lane products of a row (two chains x two lanes) as one
        // double-float, times e^{-+2 sigma a} in FP64
        auto rat_out = [&](int it, uint64_t Ah, uint64_t Al, uint64_t Bh, uint64_t Bl) {
            float h[4], l[4];
            f2_unpack(Ah, h[0], h[1]);
            f2_unpack(Al, l[0], l[1]);
            f2_unpack(Bh, h[2], h[3]);
            f2_unpack(Bl, l[2], l[3]);
            df_mul(h[0], l[0], h[1], l[1]);
            df_mul(h[2], l[2], h[3], l[3]);
            df_mul(h[0], l[0], h[2], l[2]);
            const int q = divN(it), i = it - q * N, k = q / K, kk = q - k * K;
            const bool down = down_bit(spin + k * NW, i);
            rat64[it] = (double(h[0]) + double(l[0])) * (down ? A.edn64 : A.eup64)[kk * N + i];
        };
        // two rows per pass, each as two independent half products: four
        // packed chains in flight (MP / 2 is even: MP is a multiple of 8)
        const int half = MP / 2;
        for (int it0 = htid; it0 < KK * N; it0 += 2 * HT) {
            const int it1 = it0 + HT;
            const bool two = it1 < KK * N;
            const RatRow r0 = rat_row(it0), r1 = rat_row(two ? it1 : it0);
            const uint64_t one = f2_pack(1.f, 1.f);
            uint64_t A0h = one, A0l = 0, B0h = one, B0l = 0, A1h = one, A1l = 0, B1h = one, B1l = 0;
            for (int j = 0; j < half; j += 2) {
                rat_step(A0h, A0l, r0, j);
                rat_step(B0h, B0l, r0, j + half);
                rat_step(A1h, A1l, r1, j);
                rat_step(B1h, B1l, r1, j + half);
            }
            rat_out(it0, A0h, A0l, B0h, B0l);
            if (two) rat_out(it1, A1h, A1l, B1h, B1l);
        }
    } else if (e64) {
        for (int e = htid; e < KK * MP; e += HT) {
            const int j = e - int(fdiv(unsigned(e), A.fdMP)) * MP;
            sm.t64[e] = j < M ? tanh(double(sm.th_hi[e]) + double(sm.th_lo[e])) : 0.0;
        }
        sync();
        double *rat64 = reinterpret_cast<double *>(sm.rat);  // the rat and bsig space: KK*N doubles
        for (int it = htid; it < KK * N; it += HT) {
            const int q = divN(it), i = it - q * N, k = q / K, kk = q - k * K;
            const bool down = down_bit(spin + k * NW, i);
            // sigma t = t (spin down) or -t: the sign by an integer XOR, so that a
            // factor costs one FMA and one multiply on the FP64 pipe
            const long long sgbit = down ? 0LL : (long long)0x8000000000000000ULL;
            const double *crow = A.c64 + (size_t(kk) * N + i) * M, *srow = A.s64 + (size_t(kk) * N + i) * M;
            const double *trow = sm.t64 + q * MP;
            auto st = [&](int j) { return __longlong_as_double(__double_as_longlong(trow[j]) ^ sgbit); };
            double p0 = 1.0, p1 = 1.0;
            int j = 0;
            for (; j + 1 < M; j += 2) {
                p0 *= fma(st(j), srow[j], crow[j]);
                p1 *= fma(st(j + 1), srow[j + 1], crow[j + 1]);
            }
            if (j < M) p0 *= fma(st(j), srow[j], crow[j]);
            rat64[it] = (p0 * p1) * (down ? A.edn64 : A.eup64)[kk * N + i];
        }
    } else {
        for (int it = htid; it < KK * N; it += HT) {
            const int q = divN(it), i = it - q * N, k = q / K, kk = q - k * K;
            const bool down = down_bit(spin + k * NW, i);
            const float *crow = sm.tc + (size_t(kk) * N + i) * MP;
            const float *srow = sm.ts + (size_t(kk) * N + i) * MP;
            const float *trow = sm.t + q * MP;
            // four independent partial products over 16-byte loads; padded units
            // (t = 0, c = 1, s = 0) contribute exactly 1, so MP needs no tail
            const float sg = down ? 1.f : -1.f;
            float p0 = 1.f, p1 = 1.f, p2 = 1.f, p3 = 1.f;
            for (int j = 0; j < MP; j += 4) {
                const float4 tt = *reinterpret_cast<const float4 *>(trow + j);
                const float4 ss = *reinterpret_cast<const float4 *>(srow + j);
                const float4 cc = *reinterpret_cast<const float4 *>(crow + j);
                p0 *= fmaf(sg * tt.x, ss.x, cc.x);
                p1 *= fmaf(sg * tt.y, ss.y, cc.y);
                p2 *= fmaf(sg * tt.z, ss.z, cc.z);
                p3 *= fmaf(sg * tt.w, ss.w, cc.w);
            }
            const float p = (p0 * p1) * (p2 * p3);
            sm.rat[it] = p * __ldg((down ? A.edn : A.eup) + kk * N + i);
        }
    }
    sync();
    for (int q = hw; q < KK; q += nhw) {
        double acc = 0.0;
        if (e64) {
            const double *rat64 = reinterpret_cast<const double *>(sm.rat);
            for (int i = lane; i < N; i += 32) acc += rat64[q * N + i];
            acc = warp_sum(acc);
        } else {
            float a32 = 0.f;
            for (int i = lane; i < N; i += 32) a32 += sm.rat[q * N + i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) a32 += __shfl_xor_sync(0xffffffffu, a32, o);
            acc = double(a32);
        }
        if (lane == 0) sm.Dm[q] = sm.jk[q / K] - A.h * acc;
    }
    sync();
    if (writer) {
        bool ok = true;
        for (int r = 0; r < K; r++)
            for (int cc = 0; cc < K; cc++) {
                double e = 0.0;
                for (int t = 0; t < K; t++) e = fma(sm.pinv[r * K + t], sm.Dm[t * K + cc] * sm.phi[t * K + cc], e);
                ok = ok && isfinite(e);
                A.E[s * KK + r * K + cc] = cplx{e, 0.0};
            }
        for (int k = 0; k < K; k++)
            for (int kk = 0; kk < K; kk++) sm.Bm[k * K + kk] = float(sm.pinv[k * K + kk] * sm.phi[kk * K + k]);
        if (!ok) atomicOr(A.err, kErrNonFinite);
    }
    for (int t = htid; t < K * NW; t += HT) A.spins[s * K * NW + t] = spin[t];
    sync();
    // the factors of the O row (code/rbm.cc:199-239 in closed form): tanh rows
    // T[s][k][kk][j] = tanh theta_j of configuration kk under RBM k, and
    // B[s][k][kk] = (Phi^-1)_{k,kk} Phi_{kk,k}; the signs come from the spins
    if (A.out64) {
        // O_{k,p} = sum_kk (Phi^-1)_{k,kk} Phi_{kk,k} d_p(configuration kk) in FP64, layout
        // [k][a_i | b_j | w_{i*M+j}] (code/rbm.cc:199-239). The coefficients
        // times the spin signs, bs[k][kk][i], go to the ratio space (free once
        // Dm is formed) and the coefficients themselves to Dm (free once E is
        // formed): K FMAs per entry.
        const int L = N + M + N * M;
        if (A.o_split) {
            // O stored as double-float pairs for the fused S·v: the same sums
            // formed in double-float on the FP32 pipe (products with their FMA
            // error and cross terms, TwoSum-compensated sums; ~2^-46 relative)
            // from double-float splits of the coefficients and of tanh, made once
            // per sample, instead of K FP64 FMAs per entry. The splits take the
            // ratio space (bs2), the Dm space (Dm2) and t64 in place (t2).
            float2 *bs2 = reinterpret_cast<float2 *>(sm.rat);  // K*K*N: the rat and bsig space
            float2 *t2 = reinterpret_cast<float2 *>(sm.t64);   // K*K*MP, each in its own FP64 slot
            float2 *Dm2 = reinterpret_cast<float2 *>(sm.Dm);   // K*K
            bool ok = true;
            for (int e = htid; e < KK * N; e += HT) {
                const int q = divN(e), i = e - q * N, k = q / K, kk = q - k * K;
                const double b = sm.pinv[k * K + kk] * sm.phi[kk * K + k];
                float h, l;
                ok &= df_split(down_bit(spin + kk * NW, i) ? -b : b, h, l);
                bs2[e] = make_float2(h, l);
            }
            for (int e = htid; e < KK * MP; e += HT) {  // in place: a thread converts the slots it reads
                float h, l;
                ok &= df_split(sm.t64[e], h, l);
                t2[e] = make_float2(h, l);
            }
            if (htid < KK) {  // E, the last reader of Dm, was formed before the last barrier
                float h, l;
                ok &= df_split(sm.pinv[(htid / K) * K + htid % K] * sm.phi[(htid % K) * K + htid / K], h, l);
                Dm2[htid] = make_float2(h, l);
            }
            sync();
            float2 *orow2 = reinterpret_cast<float2 *>(A.O64 + s * size_t(A.sh.P));
            for (int e = htid; e < K * L; e += HT) {
                int k = 0;
#pragma unroll
                for (int t = 1; t < K; t++) k += e >= t * L ? 1 : 0;
                const int p = e - k * L;
                float sh = 0.f, sl = 0.f;
                if (p < N) {
#pragma unroll
                    for (int kk = 0; kk < K; kk++) {
                        const float2 b = bs2[(k * K + kk) * N + p];
                        df_acc(sh, sl, b.x, b.y);
                    }
                } else if (p < N + M) {
                    const int j = p - N;
#pragma unroll
                    for (int kk = 0; kk < K; kk++) {
                        const float2 d = Dm2[k * K + kk], t = t2[(kk * K + k) * MP + j];
                        df_fma(sh, sl, d.x, d.y, t.x, t.y);
                    }
                } else {
                    const int i = int(fdiv(unsigned(p - N - M), A.fdM)), j = (p - N - M) - i * M;
#pragma unroll
                    for (int kk = 0; kk < K; kk++) {
                        const float2 b = bs2[(k * K + kk) * N + i], t = t2[(kk * K + k) * MP + j];
                        df_fma(sh, sl, b.x, b.y, t.x, t.y);
                    }
                }
                const float hi = sh + sl;
                orow2[e] = make_float2(hi, sl - (hi - sh));
                ok &= isfinite(hi);
            }
            if (!ok) atomicOr(A.err, kErrNonFinite);
            sync();
            return;
        }
        double *bs = reinterpret_cast<double *>(sm.rat);  // K*K*N doubles: the rat and bsig space
        for (int e = htid; e < KK * N; e += HT) {
            const int q = divN(e), i = e - q * N, k = q / K, kk = q - k * K;
            const double b = sm.pinv[k * K + kk] * sm.phi[kk * K + k];
            bs[e] = down_bit(spin + kk * NW, i) ? -b : b;
        }
        if (htid < KK) sm.Dm[htid] = sm.pinv[(htid / K) * K + htid % K] * sm.phi[(htid % K) * K + htid / K];
        sync();
        double *orow = A.O64 + s * size_t(A.sh.P);
        bool split_ok = true;
        for (int e = htid; e < K * L; e += HT) {
            int k = 0;
#pragma unroll
            for (int t = 1; t < K; t++) k += e >= t * L ? 1 : 0;
            const int p = e - k * L;
            double v = 0.0;
            if (p < N) {
#pragma unroll
                for (int kk = 0; kk < K; kk++) v += bs[(k * K + kk) * N + p];
            } else if (p < N + M) {
                const int j = p - N;
#pragma unroll
                for (int kk = 0; kk < K; kk++) v = fma(sm.Dm[k * K + kk], sm.t64[(kk * K + k) * MP + j], v);
            } else {
                const int i = int(fdiv(unsigned(p - N - M), A.fdM)), j = (p - N - M) - i * M;
#pragma unroll
                for (int kk = 0; kk < K; kk++) v = fma(bs[(k * K + kk) * N + i], sm.t64[(kk * K + k) * MP + j], v);
            }
            if (A.o_split) {  // as hi + lo for the fused S·v (nqes_math.cuh: df_split)
                float hi, lo;
                split_ok &= df_split(v, hi, lo);
                reinterpret_cast<float2 *>(orow)[e] = make_float2(hi, lo);
            } else {
                orow[e] = v;
            }
        }
        if (!split_ok) atomicOr(A.err, kErrNonFinite);
    } else {
        const int MT = fact_mt(M);
        float *ft = A.FT + s * size_t(KK) * MT;
        for (int e = htid; e < KK * MT; e += HT) {
            const int q = int(fdiv(unsigned(e), A.fdMT)), j = e - q * MT, k = q / K, kk = q - k * K;
            ft[e] = j < M ? sm.t[(kk * K + k) * MP + j] : 0.f;
        }
        if (htid < KK) A.FB[s * KK + htid] = sm.Bm[htid];
    }
    sync();
}

template <int K_, int U>
__global__ void __maxnreg__(U * K_ >= 16 ? 255 : NQES_DW_MAXNREG) k_sample_dw(const MixedArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int K = K_;
    const int N = A.sh.N, NW = A.sh.NW, MP = A.MP;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = T >> 5;
    const int c = blockIdx.x;
    const bool e64 = A.out64 || A.e64;  // FP64 local energies (tanh of the exact theta, FP64 tables)
    if (!dyn_smem_covers(dsmem_bytes(N, MP, K, A.stage != 0, e64)) || K * NW > kMaxSpinWords || A.G * A.U != MP) {
        if (tid == 0) atomicOr(A.err, kErrLaunch);
        return;
    }
    DSmem sm = dcarve(smem_raw, N, MP, K, e64);
    const bool writer = tid == 0;
    const size_t tb = dw_table_bytes(N, MP, K);
    if (A.stage) {
        // the step's tables into shared memory by bulk copies (one mbarrier phase)
        float *stc = sm.tabs, *sts = stc + tb / 4, *stwh = sts + tb / 4, *stwl = stwh + tb / 4;
        if (writer) {
            mbar_init(sm.mbar, 1);
            mbar_expect_tx(sm.mbar, unsigned(4 * tb));
            bool ok;
            if (A.stage_fault) {
                // test hook: the phase waits for bytes that no copy delivers
                // (nothing is in flight), under a short poll limit
                ok = mbar_wait(sm.mbar, 0, 4096);
            } else {
                bulk_g2s(stc, A.cp, unsigned(tb), sm.mbar);
                bulk_g2s(sts, A.spp, unsigned(tb), sm.mbar);
                bulk_g2s(stwh, A.whp, unsigned(tb), sm.mbar);
                bulk_g2s(stwl, A.wlp, unsigned(tb), sm.mbar);
                ok = mbar_wait(sm.mbar, 0);
            }
            sm.flag[2] = ok ? 1 : 0;
            if (!ok) atomicOr(A.err, kErrTimeout);
        }
        __syncthreads();
        if (!sm.flag[2]) return;  // every thread: the copy did not complete in time
        sm.tc = stc;
        sm.ts = sts;
        sm.twh = stwh;
        sm.twl = stwl;
    } else {
        sm.tc = A.cp;
        sm.ts = A.spp;
        sm.twh = A.whp;
        sm.twl = A.wlp;
    }

    // init_multi_spin (code/rbm.cc:98-119): every thread advances the stream;
    // warp 0 keeps it for the proposals.
    Pcg64 rng = pcg_seed(A.sp->seed + uint64_t(c));
    if (writer)
        for (int t = 0; t < K * NW; t++) sm.spin[t] = 0;
    __syncthreads();
    for (int k = 0; k < K; k++)
        for (int i = 0; i < N; i++) {
            const bool d = pcg_bernoulli_half(rng);
            if (d && writer) sm.spin[k * NW + (i >> 6)] |= 1ULL << (i & 63);
        }
    __syncthreads();
    for (int k = 0; k < K; k++) rebuild_row(A, sm, k);

    unsigned long long nacc = 0, nexact = 0;
    int rowctr = 0;
    const int total = A.burn + A.m;
    // With helper warps, a sweep's sample is formed by warps 1.. while warp 0
    // runs the first row of the next sweep (named barrier 1 among the helpers);
    // pending: that sample's index, -1 when none waits.
    const bool overlap = nwarp >= 2;
    const int HTn = T - 32;
    auto helper_sync = [HTn] { asm volatile("bar.sync 1, %0;" ::"r"(HTn) : "memory"); };
    long long pending = -1;
    for (int sw = 0; sw < total; sw++) {
        for (int k = 0; k < K; k++, rowctr++) {
            if (warp == 0) {
                const bool ch = run_row<K_, U>(A, sm, k, rng, nacc, nexact);
                if (lane == 0) sm.flag[rowctr & 1] = ch ? 1 : 0;
            } else if (pending >= 0) {
                sample_phase<K_>(A, sm, size_t(pending), sm.spin_snap, tid - 32, T - 32, helper_sync);
                pending = -1;
            }
            __syncthreads();
            if (sm.flag[rowctr & 1]) rebuild_row(A, sm, k);  // uniform after the barrier
        }
        if (sw < A.burn) continue;
        const size_t s = size_t(c) * A.m + (sw - A.burn);
        if (overlap) {
            // the helpers take this sample while warp 0 sweeps the next row: the
            // rows of Phi, theta and tanh stay as they are until that row's
            // rebuild (after the row barrier); the configurations are copied
            if (tid < K * NW) sm.spin_snap[tid] = sm.spin[tid];
            __syncthreads();
            pending = (long long)s;
        } else {
            sample_phase<K_>(A, sm, s, sm.spin, tid, T, [] { __syncthreads(); });
        }
    }
    if (overlap && warp != 0 && pending >= 0)
        sample_phase<K_>(A, sm, size_t(pending), sm.spin_snap, tid - 32, T - 32, helper_sync);
    if (writer) {
        A.accepted[c] = nacc;
        A.exact[c] = nexact;
    }
}

// Padded tables [kk][i][MP] (padding: c = 1, s = 0, w = 0, so a padded
// factor is exactly 1), theta's b as double-float [kk][MP], and per (kk, i)
// the bound record of run_row: {u (sum_j cond_j + 2M + 16),
// sum_j |s_j| / (c_j - |s_j|), max_j 1 / (c_j - |s_j|)^2, u (2 max_j cond_j + 5)}
// with c - |s| = e^{-2|w|} and cond = (c + |s|) / (c - |s|) = e^{4|w|}, each
// rounded up; after the K*N records, per RBM 2 max_j sum_i |w_ij| (float bits,
// rounded up, maximised with atomicMax over a zeroed slot).
__global__ void k_tables_dw(Shape sh, int MP, const cplx *b, const cplx *w, float *cp, float *spp, float *whp,
                            float *wlp, float *bh, float *bl, float4 *bnd, float *cpl, float *spl) {
    const size_t nr = size_t(sh.K) * sh.N;
    for (size_t r = blockIdx.x * size_t(blockDim.x) + threadIdx.x; r < nr; r += size_t(gridDim.x) * blockDim.x) {
        double sc = 0.0, s1 = 0.0, f2 = 0.0, qm = 0.0;
        for (int j = 0; j < sh.M; j++) {
            const double aw = fabs(w[r * sh.M + j].re);
            const double d = exp(-2.0 * aw), cond = exp(4.0 * aw);
            sc += cond;
            s1 += fabs(sinh(2.0 * aw)) / d;
            f2 = fmax(f2, 1.0 / (d * d));
            qm = fmax(qm, cond);
        }
        const double up = 1.0 + 1e-6, u = 0x1p-24;
        bnd[r] = make_float4(float(u * (sc + 2.0 * sh.M + 16.0) * up), float(s1 * up), float(f2 * up),
                             float(u * (2.0 * qm + 5.0) * up));
    }
    unsigned *wsum = reinterpret_cast<unsigned *>(bnd + nr);
    for (size_t r = blockIdx.x * size_t(blockDim.x) + threadIdx.x; r < size_t(sh.K) * sh.M;
         r += size_t(gridDim.x) * blockDim.x) {
        const size_t kk = r / sh.M, j = r % sh.M;
        double sw = 0.0;
        for (int i = 0; i < sh.N; i++) sw += fabs(w[(kk * sh.N + i) * sh.M + j].re);
        atomicMax(wsum + kk, __float_as_uint(float(2.0 * sw * (1.0 + 1e-6))));
    }
    const size_t n = size_t(sh.K) * sh.N * MP;
    for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < n; t += size_t(gridDim.x) * blockDim.x) {
        const int j = int(t % MP);
        const size_t ki = t / MP;  // kk*N + i
        float c = 1.f, s = 0.f, h = 0.f, l = 0.f, cl = 0.f, sl = 0.f;
        if (j < sh.M) {
            const double wv = w[ki * sh.M + j].re;
            const double cd = cosh(2.0 * wv), sd = sinh(2.0 * wv);
            c = float(cd);
            s = float(sd);
            cl = float(cd - double(c));
            sl = float(sd - double(s));
            h = float(wv);
            l = float(wv - double(h));
        }
        cp[t] = c;
        spp[t] = s;
        cpl[t] = cl;
        spl[t] = sl;
        whp[t] = h;
        wlp[t] = l;
        if (t < size_t(sh.K) * MP) {
            const int kk = int(t / MP);
            float bh0 = 0.f, bl0 = 0.f;
            if (j < sh.M) {
                const double bv = b[size_t(kk) * sh.M + j].re;
                bh0 = float(bv);
                bl0 = float(bv - double(bh0));
            }
            bh[t] = bh0;
            bl[t] = bl0;
        }
    }
}

}  // namespace
}  // namespace nqes
