// Mixed-precision Metropolis sampler, local energy and log-derivatives (real
// weights) — the precision form of code/rbm.cc:561-632 that keeps the
// reference's Markov chains.
//
// The FP64 sampler (kernels_sample.cu) spends its time in FP64 instructions,
// which on GB300 issue at ~1/64 of the FP32 rate. Here the per-proposal work
// runs in FP32: factors f_j = c - sigma t s from FP32 tables, their product,
// and the determinant update det Phi' = sum_kk r_kk e_kk g_kk. Each FP32
// quantity carries a rigorous relative-error bound (condition numbers of the
// factors, rounding of products and sums, drift of the tracked Phi), so every
// accept decision is either certain — identical to the exact one — or is
// recomputed exactly in FP64: Phi from log cosh(theta) and the ratio from
// log cosh(theta - 2 sigma w) - log cosh(theta). The chains therefore follow
// the reference's trajectories (code/rbm.cc:530-552) while almost all
// arithmetic is FP32.
//
// Exact state: theta in FP64 (one add per hidden unit per accepted flip);
// tanh(theta) in FP32 is recomputed from it, so it never drifts; a row of Phi
// is recomputed exactly from theta at the end of each row that changed. Local
// energies are formed in FP32 ratios and combined in FP64; the log-derivatives
// are written as their factors (kernels_factored.cu). This block form serves
// shapes beyond the decision-warp sampler's 32 hidden units per lane
// (kernels_sample_warp.cu).
#include <cfloat>

#include "nqes_internal.h"
#include "pcg64.cuh"

namespace nqes {

namespace {

constexpr int kUMax = 8;
constexpr int kMaxThreads = 256;
constexpr int kMaxSpinWords = 8;
constexpr float kEps = 5.9604645e-8f;  // FP32 unit roundoff 2^-24

__device__ __forceinline__ bool down_bit(const uint64_t *s, int i) { return (s[i >> 6] >> (i & 63)) & 1ULL; }
// Binary exponent of a finite float (0 for zero) from its bit pattern.
__device__ __forceinline__ int expo32(float x) {
    const int b = (__float_as_int(x) >> 23) & 0xff;
    return b == 0 ? 0 : b - 127;
}

struct MSmem {
    double *th, *phi, *pinv, *Dm, *jk, *lsum;
    float *t, *red, *rbd, *rat, *bsig, *Bm;
    uint64_t *spin;
    int *flag;
};

__host__ __device__ inline size_t msmem_bytes(int N, int M, int K) {
    const size_t KK = size_t(K) * K;
    const size_t nd = KK * M + KK + KK + KK + 4 + 32;
    const size_t nf = KK * M + 32 + 32 + 2 * KK * N + KK;
    return nd * 8 + ((nf * 4 + 7) / 8) * 8 + 8 * kMaxSpinWords + 4 * 8;
}

__device__ inline MSmem mcarve(unsigned char *base, int N, int M, int K) {
    const int KK = K * K;
    MSmem s;
    double *d = reinterpret_cast<double *>(base);
    s.th = d; d += KK * M;
    s.phi = d; d += KK;
    s.pinv = d; d += KK;
    s.Dm = d; d += KK;
    s.jk = d; d += 4;
    s.lsum = d; d += 32;
    float *f = reinterpret_cast<float *>(d);
    s.t = f; f += KK * M;
    s.red = f; f += 32;
    s.rbd = f; f += 32;
    s.rat = f; f += KK * N;
    s.bsig = f; f += KK * N;
    s.Bm = f; f += KK;
    const size_t nf = size_t(KK) * M + 32 + 32 + 2 * size_t(KK) * N + KK;
    unsigned char *p = reinterpret_cast<unsigned char *>(d) + ((nf * 4 + 7) / 8) * 8;
    s.spin = reinterpret_cast<uint64_t *>(p);
    s.flag = reinterpret_cast<int *>(s.spin + kMaxSpinWords);
    return s;
}

// log Phi[k][kk] up to a constant common to every entry, exactly in FP64:
//   sum_i sigma_i a_i + sum_j log cosh theta_j
//     = sum_i sigma_i a_i + sum_j |theta_j| + log prod_j (1 + e^{-2|theta_j|}) - M log 2,
// one exp per hidden unit and one log per entry (each factor lies in (1, 2],
// so the product stays in range for M <= 512). With a proposal (flip of spin i)
// the same for the flipped configuration, theta'_j = theta_j - 2 sigma_i w_ij.
// Warps kk < K write lsum[k*K + kk] (current) and lsum[16 + kk] (proposed).
__device__ void row_logsums(const MixedArgs &A, MSmem &sm, int k, int i, bool with_new) {
    const int N = A.sh.N, M = A.sh.M, K = A.sh.K, NW = A.sh.NW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    const bool down = with_new && down_bit(sm.spin + k * NW, i);
    for (int kk = warp; kk < K; kk += nwarp) {
        const int q = k * K + kk;
        double lin = 0.0, pr = 1.0, lin2 = 0.0, pr2 = 1.0;
        for (int j = lane; j < M; j += 32) {
            const double th = sm.th[q * M + j];
            lin += fabs(th);
            pr *= 1.0 + exp(-2.0 * fabs(th));
            if (with_new) {
                const double w = A.w64[(size_t(kk) * N + i) * M + j];
                const double th2 = down ? th + 2.0 * w : th - 2.0 * w;
                lin2 += fabs(th2);
                pr2 *= 1.0 + exp(-2.0 * fabs(th2));
            }
        }
        double as = 0.0;
        for (int i2 = lane; i2 < N; i2 += 32) as += down_bit(sm.spin + k * NW, i2) ? -A.a64[kk * N + i2] : A.a64[kk * N + i2];
        lin = warp_sum(lin);
        as = warp_sum(as);
        pr = warp_prod(pr);
        if (with_new) {
            lin2 = warp_sum(lin2);
            pr2 = warp_prod(pr2);
        }
        if (lane == 0) {
            sm.lsum[q] = as + lin + log(pr);
            if (with_new) {
                const double ai = A.a64[kk * N + i];
                sm.lsum[16 + kk] = as + (down ? 2.0 * ai : -2.0 * ai) + lin2 + log(pr2);
            }
        }
    }
}

// Exact row k of Phi from theta (FP64), scaled by the row's largest entry.
// Block-wide; starts and ends with a barrier (theta and the spins were just
// written by other threads).
__device__ void resync_row(const MixedArgs &A, MSmem &sm, int k) {
    const int K = A.sh.K;
    __syncthreads();
    row_logsums(A, sm, k, 0, false);
    __syncthreads();
    if (threadIdx.x == 0) {
        double mx = -1e308;
        for (int kk = 0; kk < K; kk++) mx = fmax(mx, sm.lsum[k * K + kk]);
        for (int kk = 0; kk < K; kk++) sm.phi[k * K + kk] = exp(sm.lsum[k * K + kk] - mx);
    }
    __syncthreads();
}

// Cofactor and absolute cofactor (products of |entries|) of a K×K matrix.
__device__ void cofactors(const double *m, int K, int r, int c, double &cof, double &cabs) {
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
    // permanent-like bound: sum of |products| of every Leibniz term
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

template <int UMAX>
__global__ void __maxnreg__(UMAX >= 4 ? 255 : 128) k_sample_mixed(const MixedArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = A.sh.N, M = A.sh.M, K = A.sh.K, NW = A.sh.NW, KK = K * K;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = T >> 5;
    const int TK = A.tk, WK = TK >> 5;
    const int my_kk = tid / TK, my_jl = tid - (tid / TK) * TK;
    const int c = blockIdx.x;
    if (!dyn_smem_covers(msmem_bytes(N, M, K)) || K * NW > kMaxSpinWords) {
        if (tid == 0) atomicOr(A.err, kErrLaunch);
        return;
    }
    MSmem sm = mcarve(smem_raw, N, M, K);
    const bool writer = tid == 0;

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
    // theta (FP64, exact) and tanh(theta) (FP32) from scratch
    for (int u = tid; u < KK * M; u += T) {
        const int q = u / M, j = u - q * M, k = q / K, kk = q - k * K;
        double th = A.b64[kk * M + j];
        for (int i = 0; i < N; i++) {
            const double w = A.w64[(size_t(kk) * N + i) * M + j];
            th = down_bit(sm.spin + k * NW, i) ? th - w : th + w;
        }
        sm.th[u] = th;
        sm.t[u] = tanhf(float(th));
    }
    __syncthreads();
    for (int k = 0; k < K; k++) resync_row(A, sm, k);

    // Decision state, identical in every warp. Lane kk < K holds the swept
    // row's Phi[k][kk] (phik) and g_kk = Phi[k][kk] cof(k, kk) in FP32, and
    // gabs32, the same product over |entries| (it bounds the effect of relative
    // errors in Phi on g). det32 is the tracked determinant with absolute error
    // bound edet; rho bounds the relative error of every tracked Phi entry,
    // summed over rows (it grows with each FP32 row update and restarts when
    // Phi is recomputed from theta).
    float phik = 0.f, g32 = 0.f, gabs32 = 0.f, det32 = 0.f, edet = 0.f, rho = 0.f;
    bool row_changed = false;
    unsigned long long nacc = 0, nexact = 0;
    auto row_setup = [&](int k) {
        if (lane < K) {
            double cof, cabs;
            cofactors(sm.phi, K, k, lane, cof, cabs);
            const double p = sm.phi[k * K + lane];
            phik = float(p);
            g32 = float(p * cof);
            gabs32 = float(fabs(p) * cabs);
        }
        row_changed = false;
    };
    // det32 and edet from an exact Phi: the FP64 determinant's own rounding is
    // bounded by 2^-50 times the sum of |Leibniz terms|.
    auto det_setup = [&]() {
        const double d = small_det(sm.phi, K);
        double perm = 0.0;
        for (int c2 = 0; c2 < K; c2++) {
            double cof, cabs;
            cofactors(sm.phi, K, 0, c2, cof, cabs);
            perm += fabs(sm.phi[c2]) * cabs;
        }
        det32 = float(d);
        edet = 4.f * kEps * fabsf(det32) + float(perm * 0x1p-50);
        rho = 0.f;
    };

    // Every row of Phi is exact (recomputed from theta) when its sweep starts:
    // rows are recomputed at the end of every row that changed.
    const int total = A.burn + A.m;
    for (int sw = 0; sw < total; sw++) {
        for (int k = 0; k < K; k++) {
            det_setup();
            row_setup(k);
            for (int i = 0; i < N; i++) {
                const int par = (i & 1) * 16;
                const bool down = down_bit(sm.spin + k * NW, i);
                const int q = k * K + my_kk;
                const float *crow = A.ch + (size_t(my_kk) * N + i) * M;
                const float *srow = A.sh32 + (size_t(my_kk) * N + i) * M;
                float prod = 1.f, eb = 0.f;
#pragma unroll
                for (int qq = 0; qq < UMAX; qq++) {
                    const int j = my_jl + qq * TK;
                    if (j < M) {
                        const float t = sm.t[q * M + j], cc = __ldg(crow + j), ss = __ldg(srow + j);
                        const float f = fmaf(down ? t : -t, ss, cc);  // c - sigma t s
                        prod *= f;
                        eb = fmaf(fabsf(cc) + 6.f * fabsf(t * ss), __frcp_rn(fabsf(f)), eb);
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    prod *= __shfl_xor_sync(0xffffffffu, prod, o);
                    eb += __shfl_xor_sync(0xffffffffu, eb, o);
                }
                if (lane == 0) {
                    sm.red[par + warp] = prod;
                    sm.rbd[par + warp] = eb;
                }
                float ea = 1.f;
                if (lane < K) ea = __ldg((down ? A.edn : A.eup) + lane * N + i);
                const uint64_t draw = pcg_next(rng);
                const float u32 = __ull2float_rn(draw) * 0x1p-64f;  // within 2 roundings of the FP64 u
                __syncthreads();
                // ---- decision, identical in every warp ----
                float r = 1.f, beta = 0.f, x = 0.f, dx = 0.f;
                if (lane < K) {
                    float ebk = 0.f;
                    for (int w2 = 0; w2 < WK; w2++) {
                        r *= sm.red[par + lane * WK + w2];
                        ebk += sm.rbd[par + lane * WK + w2];
                    }
                    // |r - exact| <= beta |r|. Per factor f = c - sigma t s: c and s
                    // rounded once from FP64, t = tanhf(float(theta)) within 5 roundings
                    // (2 ulp, and the argument's rounding times theta sech^2 / tanh <= 1),
                    // one rounding of the fma: ((|c| + 6 |t s|) / |f| + 1) u, summed
                    // in ebk without the 1; then one rounding per product. The
                    // constant covers the rounding of ebk itself and of the FP64 values.
                    beta = kEps * (ebk + 2.f * float(M) + 16.f);
                    const float re = r * ea;
                    x = re * g32;
                    // drift of Phi: every Leibniz term of g takes one entry from each
                    // row, so its relative error is at most the sum of the rows' drifts
                    dx = fabsf(re) * ((beta + 3.f * kEps) * fabsf(g32) + 1.02f * rho * gabs32) + 3.f * kEps * fabsf(x);
                }
                float s = x + __shfl_xor_sync(0xffffffffu, x, 1);
                s += __shfl_xor_sync(0xffffffffu, s, 2);
                s = __shfl_sync(0xffffffffu, s, 0);
                float ed = dx + __shfl_xor_sync(0xffffffffu, dx, 1);
                ed += __shfl_xor_sync(0xffffffffu, ed, 2);
                ed = __shfl_sync(0xffffffffu, ed, 0) * 1.01f + 4.f * kEps * fabsf(s);
                float bmax = beta;
                bmax = fmaxf(bmax, __shfl_xor_sync(0xffffffffu, bmax, 1));
                bmax = fmaxf(bmax, __shfl_xor_sync(0xffffffffu, bmax, 2));
                bmax = __shfl_sync(0xffffffffu, bmax, 0);
                bool acc = false, exact_path = false;
                {
                    const float ad = fabsf(s), lo = ad - ed, hi = ad + ed;
                    const float dd = fabsf(det32), dlo = fmaxf(dd - edet, 0.f), dhi = dd + edet;
                    const float su = u32 * (1.f + 16.f * kEps);
                    const float sl = u32 * (1.f - 16.f * kEps);
                    if (A.exact_all || !(dd > 1e-15f) || !(dd < 1e15f) || !(bmax < 0.01f)) {
                        // det == 0 (accepted, code/rbm.cc:542), squares outside the
                        // normal range or a loose bound: the exact path decides
                        exact_path = true;
                    } else if (lo > 0.f && lo * lo * (1.f - 16.f * kEps) >= su * dhi * dhi) {
                        acc = true;
                    } else if (!(hi * hi * (1.f + 16.f * kEps) < sl * dlo * dlo)) {
                        exact_path = true;  // NaN lands here as well
                    }
                }
                if (exact_path) {
                    // Exact FP64 decision. The other rows of Phi are exact (recomputed
                    // at their row's end); row k, current and proposed, from theta.
                    row_logsums(A, sm, k, i, true);
                    __syncthreads();
                    double xc = 0.0, xn = 0.0, pc = 0.0, pn = 0.0;
                    if (lane < K) {
                        double mx = -1e308;
                        for (int kk = 0; kk < K; kk++) mx = fmax(mx, sm.lsum[k * K + kk]);
                        double cof, cabs;
                        cofactors(sm.phi, K, k, lane, cof, cabs);
                        pc = exp(sm.lsum[k * K + lane] - mx);
                        pn = exp(sm.lsum[16 + lane] - mx);
                        xc = pc * cof;
                        xn = pn * cof;
                    }
                    double det_e = xc + shfl_xor(xc, 1);
                    det_e = det_e + shfl_xor(det_e, 2);
                    det_e = __shfl_sync(0xffffffffu, det_e, 0);
                    double sx = xn + shfl_xor(xn, 1);
                    sx = sx + shfl_xor(sx, 2);
                    sx = __shfl_sync(0xffffffffu, sx, 0);
                    acc = det_e == 0.0 || pcg_u01(draw) * (det_e * det_e) <= sx * sx;
                    nexact++;
                    __syncthreads();  // every warp has read Phi before row k changes
                    if (warp == 0 && lane < K) sm.phi[k * K + lane] = acc ? pn : pc;
                    __syncthreads();
                    // continue from the exact state
                    det_setup();
                    row_setup(k);
                }
                if (acc) {
                    // theta_j -= 2 sigma_i w_ij (FP64) and tanh in FP32
#pragma unroll
                    for (int qq = 0; qq < UMAX; qq++) {
                        const int j = my_jl + qq * TK;
                        if (j < M) {
                            const double w = A.w64[(size_t(my_kk) * N + i) * M + j];
                            const double th = down ? sm.th[q * M + j] + 2.0 * w : sm.th[q * M + j] - 2.0 * w;
                            sm.th[q * M + j] = th;
                            sm.t[q * M + j] = tanhf(float(th));
                        }
                    }
                    if (!exact_path) {
                        // row k of Phi times r e^{-2 sigma a}: g_kk becomes x_kk exactly
                        // as in exact arithmetic (row k's cofactors do not involve row k)
                        const float re = r * ea;
                        if (lane < K) {
                            phik *= re;
                            g32 = x;
                            gabs32 *= fabsf(re);
                        }
                        det32 = s;
                        edet = ed;
                        rho += bmax + 4.f * kEps;  // the ratio's bound and the rounding of phik
                        row_changed = true;
                    }
                    // keep the row's largest entry near 1 (exact power-of-two scaling)
                    int ex = lane < K ? expo32(phik) : -100000;
                    ex = max(ex, __shfl_xor_sync(0xffffffffu, ex, 1));
                    ex = max(ex, __shfl_xor_sync(0xffffffffu, ex, 2));
                    ex = __shfl_sync(0xffffffffu, ex, 0);
                    if (ex > 20 || ex < -20) {
                        const float sc = ldexpf(1.f, -ex);
                        phik *= sc;
                        det32 *= sc;
                        edet *= sc;
                        g32 *= sc;
                        gabs32 *= sc;
                        row_changed = true;
                    }
                    // Other warps may already read bit i+1 of this word: unchanged either way.
                    if (writer) sm.spin[k * NW + (i >> 6)] ^= 1ULL << (i & 63);
                    nacc++;
                }
            }
            // row k exact again before the next row's cofactors read it
            if (row_changed)
                resync_row(A, sm, k);
            else
                __syncthreads();
        }
        if (sw < A.burn) continue;

        // ---- sample: local energy (FP32 ratios, FP64 combination) and FP32 O ----
        const size_t s = size_t(c) * A.m + (sw - A.burn);
        if (writer) {
            double pinv[16];
            if (!small_inv(sm.phi, pinv, K)) {
                atomicOr(A.err, kErrSingular);
                for (int t = 0; t < KK; t++) pinv[t] = 0.0;
            }
            for (int t = 0; t < KK; t++) sm.pinv[t] = pinv[t];
        }
        __syncthreads();
        if (warp < K) {
            const uint64_t *sk = sm.spin + warp * NW;
            double acc = 0.0;
            for (int i = 1 + lane; i < N; i += 32) {
                const bool si = down_bit(sk, i);
                const double *Jr = A.J + size_t(i) * N;
                for (int j = 0; j < i; j++) acc += (si ^ down_bit(sk, j)) ? -Jr[j] : Jr[j];
            }
            acc = warp_sum(acc);
            if (lane == 0) sm.jk[warp] = 2.0 * acc;
        }
        for (int it = tid; it < KK * N; it += T) {
            const int q = it / N, i = it - q * N, k = q / K, kk = q - k * K;
            const bool down = down_bit(sm.spin + k * NW, i);
            const float *crow = A.ch + (size_t(kk) * N + i) * M;
            const float *srow = A.sh32 + (size_t(kk) * N + i) * M;
            const float *trow = sm.t + q * M;
            float p = 1.f;
            for (int j = 0; j < M; j++) p *= fmaf(down ? trow[j] : -trow[j], __ldg(srow + j), __ldg(crow + j));
            sm.rat[it] = p * __ldg((down ? A.edn : A.eup) + kk * N + i);
            const float B = float(sm.pinv[k * K + kk] * sm.phi[kk * K + k]);
            sm.bsig[it] = down_bit(sm.spin + kk * NW, i) ? -B : B;
        }
        __syncthreads();
        for (int q = warp; q < KK; q += nwarp) {
            float acc = 0.f;
            for (int i = lane; i < N; i += 32) acc += sm.rat[q * N + i];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) sm.Dm[q] = sm.jk[q / K] - A.h * double(acc);
        }
        __syncthreads();
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
        for (int t = tid; t < K * NW; t += T) A.spins[s * K * NW + t] = sm.spin[t];
        __syncthreads();
        // the factors of the O row (see kernels_factored.cu)
        const int MT = fact_mt(M);
        float *ft = A.FT + s * size_t(KK) * MT;
        for (int e = tid; e < KK * MT; e += T) {
            const int q = e / MT, j = e - q * MT, k = q / K, kk = q - k * K;
            ft[e] = j < M ? sm.t[(kk * K + k) * M + j] : 0.f;
        }
        if (tid < KK) A.FB[s * KK + tid] = sm.Bm[tid];
        __syncthreads();
    }
    if (writer) {
        A.accepted[c] = nacc;
        A.exact[c] = nexact;
    }
}

__global__ void k_tables_mixed(Shape sh, const cplx *a, const cplx *b, const cplx *w, float *ch, float *sh32,
                               float *eup, float *edn, double *w64, double *a64, double *b64) {
    const size_t nw = size_t(sh.K) * sh.N * sh.M;
    for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < nw; t += size_t(gridDim.x) * blockDim.x) {
        const double w2 = 2.0 * w[t].re;
        ch[t] = float(cosh(w2));
        sh32[t] = float(sinh(w2));
        w64[t] = w[t].re;
        if (t < size_t(sh.K) * sh.N) {
            eup[t] = float(exp(-2.0 * a[t].re));
            edn[t] = float(exp(2.0 * a[t].re));
            a64[t] = a[t].re;
        }
        if (t < size_t(sh.K) * sh.M) b64[t] = b[t].re;
    }
}

}  // namespace

size_t mixed_smem_bytes(const Shape &sh) { return msmem_bytes(sh.N, sh.M, sh.K); }

cudaError_t prepare_sample_mixed(const Shape &) {
    cudaError_t e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample_mixed<1>));
    if (e == cudaSuccess) e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample_mixed<2>));
    if (e == cudaSuccess) e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample_mixed<4>));
    if (e == cudaSuccess) e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample_mixed<8>));
    return e;
}

cudaError_t launch_sample_mixed(const MixedArgs &a, cudaStream_t st) {
    const size_t smem = msmem_bytes(a.sh.N, a.sh.M, a.sh.K);
    const int U = (a.sh.M + a.tk - 1) / a.tk, threads = a.sh.K * a.tk;
    if (threads > kMaxThreads || U > kUMax || a.tk % 32) return cudaErrorInvalidConfiguration;
    if (U <= 1)
        k_sample_mixed<1><<<a.chains, threads, smem, st>>>(a);
    else if (U <= 2)
        k_sample_mixed<2><<<a.chains, threads, smem, st>>>(a);
    else if (U <= 4)
        k_sample_mixed<4><<<a.chains, threads, smem, st>>>(a);
    else
        k_sample_mixed<8><<<a.chains, threads, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_tables_mixed(const Shape &sh, const cplx *a, const cplx *b, const cplx *w, float *ch, float *sh32,
                                float *eup, float *edn, double *w64, double *a64, double *b64, cudaStream_t st) {
    const size_t nw = size_t(sh.K) * sh.N * sh.M;
    const int blocks = int(std::min<size_t>((nw + 255) / 256, 4096));
    k_tables_mixed<<<blocks, 256, 0, st>>>(sh, a, b, w, ch, sh32, eup, edn, w64, a64, b64);
    return cudaGetLastError();
}

}  // namespace nqes
