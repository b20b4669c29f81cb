// Metropolis sampler, local energy and log-derivative emission — one CTA per
// Markov chain, the whole chain (start configuration, burn-in, m samples) in
// one launch. This is the GPU form of code/rbm.cc:561-632 (the chain loop of
// monte_carlo): init_multi_spin (98-119), state_fcn (146-171),
// monte_carlo_step (530-552), ising_like_hamiltonian + trapped_ion_model
// (1011-1062) and deriv (199-239).
//
// Thread layout. A chain's CTA has K*TK threads (TK a multiple of 32). Column
// block kk (RBM kk) owns threads [kk*TK, (kk+1)*TK); thread jl of the block
// owns hidden units j = jl, jl + TK, ... of that RBM. For a proposal (k, i)
// every thread forms
//     f_j = cosh(2 w_ij) - sigma_i tanh(theta_j^{(k,kk)}) sinh(2 w_ij)
// (= cosh(theta_j - 2 sigma_i w_ij) / cosh(theta_j), the factor of
// flip_state_fcn, code/rbm.cc:182-187) from per-step tables, and each warp
// multiplies its factors by shuffles. After one barrier every warp reads the
// K products and takes the accept decision itself, turning them into the new
// determinant by a Laplace expansion along row k,
//     det Phi' = sum_kk r_kk * g_kk,   g_kk = Phi[k][kk] * cofactor(k, kk),
// whose cofactors do not depend on row k and so are computed once per row and
// sweep; then the reference's acceptance test (code/rbm.cc:541-543) and, on
// acceptance, the tanh update of the thread's own units (code/rbm.cc:185).
// All warps hold identical copies of the random stream and of the decision
// state, so a proposal costs one barrier.
//
// On GB300 an FP64 warp instruction occupies the issuing warp for ~64 cycles
// whether one lane or 32 are active, so the kernel minimises the FP64
// instruction count on a proposal's critical path (factor, reduction,
// decision) rather than lane work; replicating the decision in every warp
// costs no more time than running it in one.
//
// Rows of Phi are kept scaled by exact powers of two. Every quantity the
// reference derives from Phi (the ratio |det Phi'|^2/|det Phi|^2, Phi^-1 H Phi
// and the log-derivatives) is invariant under row scaling, and power-of-two
// scaling is exact, so this changes no result while keeping Phi in range.
#include <type_traits>

#include "nqes_internal.h"
#include "pcg64.cuh"

namespace nqes {

namespace {

constexpr int kUMax = 8;          // hidden units per unit thread
constexpr int kMaxSpinWords = 8;  // K <= 4 configurations of <= 128 spins
constexpr int kMaxThreads = 256;  // K*TK threads

__device__ __forceinline__ double ldg(const double *p) { return __ldg(p); }
__device__ __forceinline__ cplx ldg(const cplx *p) {
    double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    return cplx{v.x, v.y};
}
__device__ __forceinline__ bool spin_down(const uint64_t *s, int i) { return (s[i >> 6] >> (i & 63)) & 1ULL; }
template <class S> __device__ __forceinline__ S neg_if(S v, bool n) { return n ? -v : v; }
template <class S> __device__ __forceinline__ S wt(const cplx &z);
template <> __device__ __forceinline__ double wt<double>(const cplx &z) { return z.re; }
template <> __device__ __forceinline__ cplx wt<cplx>(const cplx &z) { return z; }
__device__ __forceinline__ double rcp(double x) { return __drcp_rn(x); }
__device__ __forceinline__ cplx rcp(cplx x) {
    const double d = __drcp_rn(fma(x.re, x.re, x.im * x.im));
    return {x.re * d, -x.im * d};
}
__device__ __forceinline__ double shfl0(double v) { return __shfl_sync(0xffffffffu, v, 0); }
__device__ __forceinline__ cplx shfl0(cplx v) {
    return {__shfl_sync(0xffffffffu, v.re, 0), __shfl_sync(0xffffffffu, v.im, 0)};
}

// det == 0 and a <= b (a, b >= 0) on the bit patterns: the same answers as the
// FP64 compares (a NaN compares false), without FP64 instructions.
__device__ __forceinline__ bool zero_bits(double v) { return (__double_as_longlong(v) << 1) == 0; }
__device__ __forceinline__ bool zero_bits(const cplx &v) { return zero_bits(v.re) && zero_bits(v.im); }
__device__ __forceinline__ bool le_nonneg(double a, double b) {
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const long long nan = 0x7FF0000000000000LL;
    if ((ia & 0x7FFFFFFFFFFFFFFFLL) > nan || (ib & 0x7FFFFFFFFFFFFFFFLL) > nan) return false;
    return ia <= ib;
}

// Multiply v by 2^-e where e is v's binary exponent when it leaves [-256, 256].
template <class S> __device__ __forceinline__ void renorm(S &v, int &e) {
    int x = expo(v);
    if (x > 256 || x < -256) {
        v = scale2(v, -x);
        e += x;
    }
}

// Signed cofactor (-1)^{r+c} det(Phi without row r and column c), K <= 4.
template <class S> __device__ S cofactor(const S *m, int K, int r, int c) {
    if (K == 1) return one<S>();
    S sub[9];
    int t = 0;
    for (int a = 0; a < K; a++) {
        if (a == r) continue;
        for (int b = 0; b < K; b++)
            if (b != c) sub[t++] = m[a * K + b];
    }
    const S d = small_det(sub, K - 1);
    return ((r + c) & 1) ? -d : d;
}

template <class S> struct Smem {
    S *tnh, *phi, *pinv, *red, *rat, *bsig, *Bm, *Dm, *pm;
    double *jk, *jpart;
    int *pe, *rowe, *flag;
    uint64_t *spin;
    float *t32, *red32, *rbd32;  // rejection filter: FP32 tanh(theta), per-warp products and bounds
};

__host__ __device__ inline size_t smem_bytes(int N, int M, int K, size_t ssz) {
    size_t KK = size_t(K) * K;
    size_t nS = KK * M + 2 * KK + 32 + 2 * KK * N + 2 * KK + KK + 32;
    return nS * ssz + 8 * 4 + 8 * 32 + 8 * kMaxSpinWords + 4 * (32 + 4 + 4) + 4 * (KK * M + 64);
}

template <class S> __device__ inline Smem<S> carve(unsigned char *base, int N, int M, int K) {
    Smem<S> s;
    const int KK = K * K;
    S *p = reinterpret_cast<S *>(base);
    s.tnh = p; p += KK * M;
    s.phi = p; p += KK;
    s.pinv = p; p += KK;
    s.red = p; p += 32;
    s.rat = p; p += KK * N;
    s.bsig = p; p += KK * N;
    s.Bm = p; p += KK;
    s.Dm = p; p += KK;
    s.pm = p; p += KK + 32;  // (mantissa of Phi entries during init) + per-warp scratch
    double *d = reinterpret_cast<double *>(p);
    s.jk = d; d += 4;
    s.jpart = d; d += 32;
    s.spin = reinterpret_cast<uint64_t *>(d);
    int *ip = reinterpret_cast<int *>(s.spin + kMaxSpinWords);
    s.pe = ip; ip += 32;
    s.rowe = ip; ip += 4;
    s.flag = ip; ip += 4;
    float *fp = reinterpret_cast<float *>(ip);
    s.t32 = fp; fp += KK * M;
    s.red32 = fp; fp += 32;
    s.rbd32 = fp;
    return s;
}

// Phi and tanh(theta) from scratch for the current configuration
// (code/rbm.cc:146-171), with Phi's rows rescaled by powers of two.
template <class S>
__device__ void init_state(const SampleArgs<S> &A, Smem<S> &sm) {
    const int N = A.sh.N, M = A.sh.M, K = A.sh.K, NW = A.sh.NW, KK = K * K;
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = T >> 5;
    for (int q = 0; q < KK; q++) {
        const int k = q / K, kk = q - k * K;
        const uint64_t *sk = sm.spin + k * NW;
        S prod = one<S>();
        int pe = 0;
        for (int j = tid; j < M; j += T) {
            S th = wt<S>(A.b[kk * M + j]);
            const cplx *wc = A.w + size_t(kk) * N * M + j;
            for (int i = 0; i < N; i++) {
                S wij = wt<S>(wc[size_t(i) * M]);
                th = spin_down(sk, i) ? th - wij : th + wij;
            }
            sm.tnh[q * M + j] = ctanh_(th);
            prod = prod * ccosh_(th);
            renorm(prod, pe);
        }
        // exp(sum_i sigma_i a_i) from thread 0
        if (tid == 0) {
            S sa = zero<S>();
            for (int i = 0; i < N; i++) {
                S ai = wt<S>(A.a[kk * N + i]);
                sa = spin_down(sk, i) ? sa - ai : sa + ai;
            }
            prod = prod * cexp_(sa);
            renorm(prod, pe);
        }
        // block product of (mantissa, exponent)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            S p2 = shfl_xor(prod, o);
            int e2 = __shfl_xor_sync(0xffffffffu, pe, o);
            prod = prod * p2;
            pe += e2;
            renorm(prod, pe);
        }
        if (lane == 0) {
            sm.red[warp] = prod;
            sm.pe[warp] = pe;
        }
        __syncthreads();
        if (tid == 0) {
            S p = sm.red[0];
            int e = sm.pe[0];
            for (int w2 = 1; w2 < nwarp; w2++) {
                p = p * sm.red[w2];
                e += sm.pe[w2];
                renorm(p, e);
            }
            sm.pm[q] = p;
            sm.pe[32 - 1 - q] = e;  // exponents kept at the top of the scratch
        }
        __syncthreads();
    }
    if (tid == 0) {
        for (int k = 0; k < K; k++) {
            int emax = -100000;
            for (int kk = 0; kk < K; kk++) {
                const int q = k * K + kk;
                if (!is_zero(sm.pm[q])) emax = max(emax, sm.pe[31 - q] + expo(sm.pm[q]));
            }
            if (emax == -100000) emax = 0;
            for (int kk = 0; kk < K; kk++) {
                const int q = k * K + kk;
                sm.phi[q] = scale2(sm.pm[q], sm.pe[31 - q] - emax);
            }
            sm.rowe[k] = emax;
        }
    }
    __syncthreads();
}

// Correlation-function contributions of one sample (code/rbm.cc:730-826): for
// every site i the K×K matrices Phi^-1 F_i with F_i = Phi(flip i in every row)
// (sigma^x_i) and F_i = diag(sigma_i) Phi (sigma^z_i), and for every pair
// (i, j) Phi(flip i and j) (sigma^x_i sigma^x_j) and diag(sigma_i sigma_j) Phi
// (sigma^z_i sigma^z_j), accumulated into the chain's slice of A.corr.
// Single-flip ratios come from sm.rat (the local-energy terms); pair ratios
// use cosh(d_i + d_j) - tanh(theta) sinh(d_i + d_j) with d = 2 sigma w.
template <class S> __device__ void corr_sample(const SampleArgs<S> &A, Smem<S> &sm, int c) {
    const int N = A.sh.N, M = A.sh.M, K = A.sh.K, NW = A.sh.NW, KK = K * K;
    const int T = blockDim.x, tid = threadIdx.x;
    S *acc = A.corr + size_t(c) * A.corr_stride;
    S *ax = acc, *az = ax + size_t(N) * KK, *axx = az + size_t(N) * KK, *azz = axx + size_t(N) * N * KK;
    S *R = A.corr_scratch + size_t(c) * N * N * KK;
    for (int i = tid; i < N; i += T) {
        for (int r = 0; r < K; r++)
            for (int cc = 0; cc < K; cc++) {
                S mx = zero<S>(), mz = zero<S>();
                for (int t = 0; t < K; t++) {
                    const S pt = sm.phi[t * K + cc];
                    mx = mad(sm.pinv[r * K + t], pt * sm.rat[(t * K + cc) * N + i], mx);
                    mz = mad(sm.pinv[r * K + t], spin_down(sm.spin + t * NW, i) ? -pt : pt, mz);
                }
                ax[i * KK + r * K + cc] = ax[i * KK + r * K + cc] + mx;
                az[i * KK + r * K + cc] = az[i * KK + r * K + cc] + mz;
            }
    }
    // pair ratios R[(i*N+j)*KK + k*K+kk], i < j
    for (int it = tid; it < N * N * KK; it += T) {
        const int q = it % KK, ij = it / KK, i = ij / N, j = ij - i * N;
        if (i >= j) continue;
        const int k = q / K, kk = q - k * K;
        const bool di = spin_down(sm.spin + k * NW, i), dj = spin_down(sm.spin + k * NW, j);
        const S *ci = A.tab.ch + (size_t(kk) * N + i) * M, *si = A.tab.sh + (size_t(kk) * N + i) * M;
        const S *cj = A.tab.ch + (size_t(kk) * N + j) * M, *sj = A.tab.sh + (size_t(kk) * N + j) * M;
        const S *tr = sm.tnh + q * M;
        S p = one<S>();
        for (int l = 0; l < M; l++) {
            const S Ci = ldg(ci + l), Cj = ldg(cj + l);
            const S Si = neg_if(ldg(si + l), di), Sj = neg_if(ldg(sj + l), dj);  // sinh(d) = sigma S
            const S chs = mad(Ci, Cj, Si * Sj);
            const S shs = mad(Si, Cj, Ci * Sj);
            p = p * mad(-tr[l], shs, chs);
        }
        p = p * ldg((di ? A.tab.edn : A.tab.eup) + kk * N + i) * ldg((dj ? A.tab.edn : A.tab.eup) + kk * N + j);
        R[size_t(ij) * KK + q] = p;
    }
    __syncthreads();
    for (int ij = tid; ij < N * N; ij += T) {
        const int i = ij / N, j = ij - i * N;
        if (i > j) continue;
        for (int r = 0; r < K; r++)
            for (int cc = 0; cc < K; cc++) {
                S mxx = zero<S>(), mzz = zero<S>();
                if (i == j) {  // flipping i twice, and sigma_i^2 = 1: the identity
                    mxx = mzz = (r == cc) ? one<S>() : zero<S>();
                } else {
                    for (int t = 0; t < K; t++) {
                        const S pt = sm.phi[t * K + cc];
                        mxx = mad(sm.pinv[r * K + t], pt * R[size_t(ij) * KK + t * K + cc], mxx);
                        const bool flip = spin_down(sm.spin + t * NW, i) ^ spin_down(sm.spin + t * NW, j);
                        mzz = mad(sm.pinv[r * K + t], flip ? -pt : pt, mzz);
                    }
                }
                const size_t e1 = size_t(i * N + j) * KK + r * K + cc, e2 = size_t(j * N + i) * KK + r * K + cc;
                axx[e1] = axx[e1] + mxx;
                azz[e1] = azz[e1] + mzz;
                if (i != j) {
                    axx[e2] = axx[e2] + mxx;
                    azz[e2] = azz[e2] + mzz;
                }
            }
    }
}

// Rejection filter (FILT, real arithmetic). Most proposals are rejected, and a
// rejection changes no state, so the FP64 work of a proposal is needed only
// when it might be accepted. Each proposal is first evaluated in FP32 from
// FP32 roundings of the FP64 tables and of tanh(theta), with a rigorous bound
// on its distance from the FP64 value:
//   factor f = c - sigma t s: c, s, t and the fma each rounded once, so
//     |f32 - f| <= (2 cond + 1) u |f|,  cond = (|c| + |t s|) / |f|;
//   product r of the M factors: sum of the factors' bounds plus one rounding
//     per product, beta = u (3 sum cond + 2M + 16) with slack for the FP64
//     value's own rounding;
//   x_kk = r e^{-2 sigma a} g_kk and det' = sum_kk x_kk: four more roundings
//     per term and K for the sum, |det'32 - det'64| <= 1.02 sum beta |x| +
//     (8 + K) u sum |x| (1.02 turns bounds relative to the FP64 values into
//     bounds relative to the computed ones while beta < 0.01).
// When (|det'32| + bound)^2 < u |det|^2 with a margin for the roundings of
// the comparison itself, the FP64 test u |det|^2 <= |det'|^2 fails for
// certain and the proposal is rejected without FP64 work. Every other
// proposal runs the FP64 code unchanged, so the chains, Phi, tanh(theta) and
// all results are bit-identical to the unfiltered kernel. The filter's
// determinant and g_kk are FP32 copies scaled by 2^-expo(det) so that
// |det|^2 stays within FP32 range; det == 0, non-finite values, FP32 over-
// or underflow and large bounds all fall through to FP64.
constexpr float kU32 = 5.9604645e-8f;  // FP32 unit roundoff 2^-24

template <class S, int UMAX, bool FILT, bool HEIS>
__global__ void __maxnreg__(UMAX >= 4 ? 255 : 128) k_sample(const SampleArgs<S> A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int N = A.sh.N, M = A.sh.M, K = A.sh.K, NW = A.sh.NW, KK = K * K, L = A.sh.L;
    const size_t P = size_t(A.sh.P);
    const int T = blockDim.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nwarp = T >> 5;
    const int TK = A.tk, WK = TK >> 5;
    const int my_kk = tid / TK, my_jl = tid - (tid / TK) * TK;
    const int c = blockIdx.x;
    if (!dyn_smem_covers(smem_bytes(N, M, K, sizeof(S))) || K * NW > kMaxSpinWords) {
        if (tid == 0) atomicOr(A.err, kErrLaunch);
        return;
    }
    Smem<S> sm = carve<S>(smem_raw, N, M, K);

    // Every thread advances an identical copy of the chain's pcg64 stream, so
    // each warp holds every draw and takes every accept decision itself.
    Pcg64 rng{0, 0};
    if (A.cfg) {
        for (int t = tid; t < K * NW; t += T) sm.spin[t] = A.cfg[size_t(c) * K * NW + t];
    } else {
        // init_multi_spin: K·N Bernoulli draws, k-major (code/rbm.cc:98-119).
        rng = pcg_seed(A.sp->seed + uint64_t(c));
        if (tid == 0)
            for (int t = 0; t < K * NW; t++) sm.spin[t] = 0;
        __syncthreads();
        for (int k = 0; k < K; k++)
            for (int i = 0; i < N; i++) {
                const bool d = pcg_bernoulli_half(rng);
                if (d && tid == 0) sm.spin[k * NW + (i >> 6)] |= 1ULL << (i & 63);
            }
    }
    __syncthreads();
    init_state(A, sm);

    // Decision state, identical in every warp: det Phi, |det Phi|^2 and, in
    // lanes kk < K, the current row's Phi[k][kk] and g_kk = Phi[k][kk] cof(k, kk).
    S det = zero<S>(), g = zero<S>(), phik = zero<S>();
    double detn = 0.0;
    unsigned long long nacc = 0;
    // Filter copies, identical in every thread: g_kk / 2^e and (det / 2^e)^2, e = expo(det).
    float g32[4] = {0.f, 0.f, 0.f, 0.f}, dn32 = 0.f;
    auto filt_setup = [&]() {
        if constexpr (FILT) {
            const int e = is_zero(det) ? 0 : expo(det);
            const double ds = scale2(det, -e);
            dn32 = float(ds * ds);
#pragma unroll
            for (int kk = 0; kk < 4; kk++)
                if (kk < K) g32[kk] = float(scale2(__shfl_sync(0xffffffffu, g, kk), -e));
        }
    };
    // The filter pays when most proposals are rejected: a sweep runs it when
    // the chain's previous sweep accepted fewer than half of its proposals
    // (a count every thread holds, so the choice is uniform in the CTA).
    bool filt_next = FILT;
    unsigned long long nacc_sweep = 0;
    const bool writer = tid == 0;  // the one thread that commits shared state

    const int total = A.cfg ? 1 : A.burn + A.m;
    for (int sw = 0; sw < total; sw++) {
        if (!A.cfg) {
            // ---- one sweep: proposals k outer, i inner (code/rbm.cc:536-551) ----
            det = small_det(sm.phi, K);  // recomputed at every sweep, as code/rbm.cc:533
            detn = norm2(det);
            const bool use_f = filt_next;
            if constexpr (FILT) {
                if (use_f) {
                    for (int t = tid; t < KK * M; t += T) sm.t32[t] = float(sm.tnh[t]);
                    __syncthreads();
                }
                nacc_sweep = nacc;
            }
            for (int k = 0; k < K; k++) {
                if (lane < K) {
                    phik = sm.phi[k * K + lane];
                    g = phik * cofactor(sm.phi, K, k, lane);
                }
                if (use_f) filt_setup();
                S *trow = sm.tnh + (k * K + my_kk) * M;
                for (int i = 0; i < N; i++) {
                    const int par = (i & 1) * 16;  // reduction slots alternate between proposals
                    const bool down = spin_down(sm.spin + k * NW, i);
                    const S *crow = A.tab.ch + (size_t(my_kk) * N + i) * M;
                    const S *srow = A.tab.sh + (size_t(my_kk) * N + i) * M;
                    S tq[UMAX], cq[UMAX], sq[UMAX], fq[UMAX];
                    uint64_t draw = 0;
                    bool loaded = false;
                    if (FILT && use_f) {
                        // ---- FP32 stage: certain rejections skip the FP64 stage ----
                        loaded = true;
                        const float *c32 = A.c32 + (size_t(my_kk) * N + i) * M;
                        const float *s32 = A.s32 + (size_t(my_kk) * N + i) * M;
                        const float *t32 = sm.t32 + (k * K + my_kk) * M;
                        float p32 = 1.f, eb = 0.f;
#pragma unroll
                        for (int q = 0; q < UMAX; q++) {
                            const int j = my_jl + q * TK;
                            if (j < M) {
                                const float t = t32[j], cc = __ldg(c32 + j), ss = __ldg(s32 + j);
                                const float f = fmaf(down ? t : -t, ss, cc);
                                p32 *= f;
                                eb = fmaf(fabsf(cc) + fabsf(t * ss), __frcp_rn(fabsf(f)), eb);
                                // operands of the FP64 stage, loaded while the filter runs
                                tq[q] = trow[j];
                                cq[q] = ldg(crow + j);
                                sq[q] = ldg(srow + j);
                            }
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            p32 *= __shfl_xor_sync(0xffffffffu, p32, o);
                            eb += __shfl_xor_sync(0xffffffffu, eb, o);
                        }
                        if (lane == 0) {
                            sm.red32[par + warp] = p32;
                            sm.rbd32[par + warp] = eb;
                        }
                        float ea32[4];
#pragma unroll
                        for (int kk = 0; kk < 4; kk++)
                            ea32[kk] = kk < K ? __ldg((down ? A.ed32 : A.eu32) + kk * N + i) : 0.f;
                        draw = pcg_next(rng);
                        const float ud32 = __ull2float_rn(draw) * 0x1p-64f * dn32;
                        __syncthreads();
                        float sx = 0.f, sab = 0.f, eterm = 0.f, bmax = 0.f;
#pragma unroll
                        for (int kk = 0; kk < 4; kk++) {
                            if (kk < K) {
                                float r = sm.red32[par + kk * WK], e2 = sm.rbd32[par + kk * WK];
                                for (int w2 = 1; w2 < WK; w2++) {
                                    r *= sm.red32[par + kk * WK + w2];
                                    e2 += sm.rbd32[par + kk * WK + w2];
                                }
                                const float beta = kU32 * (3.f * e2 + 2.f * float(M) + 16.f);
                                const float xx = r * ea32[kk] * g32[kk];
                                sx += xx;
                                sab += fabsf(xx);
                                eterm = fmaf(beta, fabsf(xx), eterm);
                                bmax = fmaxf(bmax, beta);
                            }
                        }
                        const float hi = fabsf(sx) + 1.02f * eterm + (8.f + float(K)) * kU32 * sab;
                        if (bmax < 0.01f && ud32 > 1e-30f && ud32 < 1e30f &&
                            hi * hi * (1.f + 4.f * kU32) < ud32 * (1.f - 8.f * kU32))
                            continue;  // rejected: no state changes (same in every thread)
                    }
                    // ---- FP64 stage (the whole proposal when unfiltered) ----
                    S prod = one<S>();
#pragma unroll
                    for (int q = 0; q < UMAX; q++) {
                        const int j = my_jl + q * TK;
                        if (j < M) {
                            if (!loaded) {
                                tq[q] = trow[j];
                                cq[q] = ldg(crow + j);
                                sq[q] = ldg(srow + j);
                            }
                            // f = cosh(ws) - tanh * sinh(ws), ws = 2 sigma w
                            fq[q] = mad(neg_if(tq[q], !down), sq[q], cq[q]);
                            prod = q == 0 ? fq[q] : prod * fq[q];
                        }
                    }
                    prod = warp_prod(prod);
                    if (lane == 0) sm.red[par + warp] = prod;
                    // e^{-2 sigma_i a_i} g_kk and u |det Phi|^2 while the other warps finish
                    S ea = one<S>(), eg = zero<S>();
                    if (lane < K) {
                        ea = ldg((down ? A.tab.edn : A.tab.eup) + lane * N + i);
                        eg = ea * g;
                    }
                    // u from the draw with integer instructions, one FP64 multiply
                    const uint64_t dr = loaded ? draw : pcg_next(rng);
                    const double ud = __longlong_as_double(static_cast<long long>(pcg_u01_bits(dr))) * detn;
                    __syncthreads();
                    // det Phi' = sum_kk r_kk e^{-2 sigma a} g_kk over lanes 0..K-1 (K <= 4)
                    S x = zero<S>(), r = one<S>();
                    if (lane < K) {
                        r = sm.red[par + lane * WK];
                        for (int w2 = 1; w2 < WK; w2++) r = r * sm.red[par + lane * WK + w2];
                        x = r * eg;
                    }
                    S s = x + shfl_xor(x, 1);
                    s = s + shfl_xor(s, 2);
                    s = shfl0(s);
                    const double np = norm2(s);
                    // Accept iff u <= min(1, |det Phi'|^2 / |det Phi|^2), with
                    // probability one when det Phi == 0 (code/rbm.cc:541-543),
                    // evaluated as u |det Phi|^2 <= |det Phi'|^2.
                    const bool acc = zero_bits(det) || le_nonneg(ud, np);
                    if (acc) {
                        // tanh' = (tanh cosh(ws) - sinh(ws)) / f  (code/rbm.cc:185)
#pragma unroll
                        for (int q = 0; q < UMAX; q++) {
                            const int j = my_jl + q * TK;
                            if (j < M) {
                                trow[j] = mad(tq[q], cq[q], neg_if(sq[q], !down)) * rcp(fq[q]);
                                if constexpr (FILT)
                                    if (use_f) sm.t32[(k * K + my_kk) * M + j] = float(trow[j]);
                            }
                        }
                        if (lane < K) {
                            g = x;
                            phik = phik * (r * ea);
                        }
                        det = s;
                        detn = np;
                        int ex = lane < K ? expo(phik) : -100000;
                        ex = max(ex, __shfl_xor_sync(0xffffffffu, ex, 1));
                        ex = max(ex, __shfl_xor_sync(0xffffffffu, ex, 2));
                        ex = __shfl_sync(0xffffffffu, ex, 0);
                        if (ex > 256 || ex < -256) {
                            phik = scale2(phik, -ex);
                            g = scale2(g, -ex);
                            det = scale2(det, -ex);
                            detn = norm2(det);
                            if (writer) sm.rowe[k] += ex;
                        }
                        if (use_f) filt_setup();
                        if (warp == 0 && lane < K) sm.phi[k * K + lane] = phik;
                        // Other warps may already read bit i+1 of this word: the
                        // read sees bit i+1 unchanged before or after the flip.
                        if (writer) sm.spin[k * NW + (i >> 6)] ^= 1ULL << (i & 63);
                        nacc++;
                    }
                }
                __syncthreads();
            }
            if constexpr (FILT) filt_next = (nacc - nacc_sweep) * 2 < (unsigned long long)(K * N);
            if (sw < A.burn) continue;
        }
        // ---- sample: local energy and log-derivatives ----
        const size_t s = A.cfg ? size_t(c) : size_t(c) * A.m + (sw - A.burn);
        __syncthreads();
        if (tid == 0) {
            if (!small_inv(sm.phi, sm.pinv, K)) {
                // Sampling stops with an error; an evaluation at given
                // configurations (e.g. two equal rows) leaves E and O to
                // k_eval_singular (the pseudo-inverse; O is zero, the
                // determinants det(Phi^+ Phi~) of a rank-deficient product).
                atomicOr(A.err, kErrSingular);
                for (int t = 0; t < KK; t++) sm.pinv[t] = zero<S>();
            }
        }
        __syncthreads();
        {
            // J(s_k) = 2 sum_{i>j} J_ij sigma_i sigma_j (code/rbm.cc:1011-1031): the
            // N x N grid strided over the block, partial sums per warp, then the
            // warps' partials in warp order (deterministic); jk is complete after
            // the barrier below
            double acc[4] = {0.0, 0.0, 0.0, 0.0};
            int i = tid / N, j = tid - (tid / N) * N;
            const int di = T / N, dj = T - (T / N) * N;
            while (i < N) {
                if (j < i) {
                    const double p = A.J[size_t(i) * N + j];
#pragma unroll
                    for (int k = 0; k < 4; k++)
                        if (k < K) acc[k] += (spin_down(sm.spin + k * NW, i) ^ spin_down(sm.spin + k * NW, j)) ? -p : p;
                }
                j += dj;
                i += di;
                if (j >= N) {
                    j -= N;
                    i++;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (k < K) {
                    acc[k] = warp_sum(acc[k]);
                    if (lane == 0) sm.jpart[warp * 4 + k] = acc[k];
                }
        }
        // Ratios Phi(flip i in row k)[k][kk] / Phi[k][kk] for every (k, kk, i),
        // the N single-flip terms of the transverse field (code/rbm.cc:1050-1058)
        // and the x observables of the correlation pass.
        const bool single = !HEIS || A.corr;
        for (int it = tid; it < KK * N; it += T) {
            const int q = it / N, i = it - q * N, k = q / K, kk = q - k * K;
            if (single) {
                const bool down = spin_down(sm.spin + k * NW, i);
                const S *crow = A.tab.ch + (size_t(kk) * N + i) * M;
                const S *srow = A.tab.sh + (size_t(kk) * N + i) * M;
                const S *trow = sm.tnh + q * M;
                S p = one<S>();
                for (int j = 0; j < M; j++) p = p * mad(neg_if(trow[j], !down), ldg(srow + j), ldg(crow + j));
                sm.rat[it] = p * ldg((down ? A.tab.edn : A.tab.eup) + kk * N + i);
            }
            // B(kk->k) sigma^{(kk)}_i for the a and w derivatives, where
            // B(kk->k) = (Phi^-1)[k][kk] Phi[kk][k] (closed form of the
            // determinants in code/rbm.cc:211-236).
            const S B = sm.pinv[k * K + kk] * sm.phi[kk * K + k];
            sm.bsig[it] = spin_down(sm.spin + kk * NW, i) ? -B : B;
        }
        __syncthreads();
        if (A.corr) {  // correlation pass: observables instead of E and O
            corr_sample(A, sm, c);
            __syncthreads();
            continue;
        }
        if (tid < K) {
            double jt = 0.0;
            for (int w2 = 0; w2 < nwarp; w2++) jt += sm.jpart[w2 * 4 + tid];
            sm.jk[tid] = HEIS ? A.delta * jt : 2.0 * jt;
        }
        __syncthreads();
        if constexpr (!HEIS) {
            for (int q = warp; q < KK; q += nwarp) {
                S acc = zero<S>();
                for (int i = lane; i < N; i += 32) acc = acc + sm.rat[q * N + i];
                acc = warp_sum(acc);
                if (lane == 0) {
                    sm.Dm[q] = one<S>() * sm.jk[q / K] - A.h * acc;
                    if (A.dm_out) A.dm_out[s * KK + q] = to_c(sm.Dm[q]);
                }
            }
        } else {
            // Heisenberg-like (code/rbm.cc:1091-1119): for each pair i > j with
            // J_ij != 0 and spins i, j of row k anti-aligned, the two-flip ratio
            // Phi(flip i, j)[k][kk] / Phi[k][kk] = e^{-2 s_i a_i - 2 s_j a_j}
            // prod_m [cosh(d_i + d_j) - tanh(theta_m) sinh(d_i + d_j)],
            // d = 2 s w_{.m}, each factor formed as c_i (c_j - t u_j) + u_i (u_j - t c_j)
            // from the per-step tables (c = cosh 2w, u = s sinh 2w); D_k =
            // delta sum_{i>j} J_ij s_i s_j + 2 sum_{anti-aligned} J_ij ratio.
            // Per (k, kk): the pairs strided over the block, per-warp partials
            // added in warp order (deterministic).
            for (int q = 0; q < KK; q++) {
                const int k = q / K, kk = q - k * K;
                const uint64_t *sk = sm.spin + k * NW;
                const S *trow = sm.tnh + q * M;
                S acc = zero<S>();
                for (int pr = tid; pr < N * N; pr += T) {
                    const int i = pr / N, j = pr - (pr / N) * N;
                    if (j >= i) continue;
                    const double p = A.J[size_t(i) * N + j];
                    const bool di = spin_down(sk, i), dj = spin_down(sk, j);
                    if (p == 0.0 || di == dj) continue;
                    const S *ci = A.tab.ch + (size_t(kk) * N + i) * M, *si = A.tab.sh + (size_t(kk) * N + i) * M;
                    const S *cj = A.tab.ch + (size_t(kk) * N + j) * M, *sj = A.tab.sh + (size_t(kk) * N + j) * M;
                    S r = one<S>();
                    for (int m = 0; m < M; m++) {
                        const S t = trow[m], c1 = ldg(ci + m), c2 = ldg(cj + m);
                        const S u1 = neg_if(ldg(si + m), di), u2 = neg_if(ldg(sj + m), dj);
                        r = r * mad(c1, mad(neg_if(t, true), u2, c2), u1 * mad(neg_if(t, true), c2, u2));
                    }
                    r = r * ldg((di ? A.tab.edn : A.tab.eup) + kk * N + i) * ldg((dj ? A.tab.edn : A.tab.eup) + kk * N + j);
                    acc = mad(one<S>() * (2.0 * p), r, acc);
                }
                acc = warp_sum(acc);
                if (lane == 0) sm.red[warp] = acc;
                __syncthreads();
                if (tid == 0) {
                    S tot = zero<S>();
                    for (int w2 = 0; w2 < nwarp; w2++) tot = tot + sm.red[w2];
                    sm.Dm[q] = one<S>() * sm.jk[k] + tot;
                    if (A.dm_out) A.dm_out[s * KK + q] = to_c(sm.Dm[q]);
                }
                __syncthreads();
            }
        }
        __syncthreads();
        if (tid == 0) {
            // E = Phi^-1 (D o Phi)  (code/rbm.cc:1046-1061)
            bool ok = true;
            for (int r = 0; r < K; r++)
                for (int cc = 0; cc < K; cc++) {
                    S e = zero<S>();
                    for (int t = 0; t < K; t++) e = mad(sm.pinv[r * K + t], sm.Dm[t * K + cc] * sm.phi[t * K + cc], e);
                    ok = ok && finite(e);
                    A.E[s * KK + r * K + cc] = to_c(e);
                }

            for (int k = 0; k < K; k++)
                for (int kk = 0; kk < K; kk++) sm.Bm[k * K + kk] = sm.pinv[k * K + kk] * sm.phi[kk * K + k];
            if (!ok) atomicOr(A.err, kErrNonFinite);
        }
        for (int t = tid; t < K * NW; t += T) A.spins[s * K * NW + t] = sm.spin[t];
        if (A.cfg && A.phi_out) {
            for (int t = tid; t < KK; t += T) A.phi_out[s * KK + t] = to_c(scale2(sm.phi[t], sm.rowe[t / K]));
            for (int t = tid; t < KK * M; t += T) {
                const int q = t / M, j = t - q * M;
                A.tanh_out[s * KK * M + size_t(j) * KK + q] = to_c(sm.tnh[t]);
            }
        }
        __syncthreads();
        // O row, layout [k][a_i | b_j | w_{i*M+j}] (code/rbm.cc:199-239):
        //   O_{k,a_i}  = sum_kk B(kk->k) sigma^{(kk)}_i
        //   O_{k,b_j}  = sum_kk B(kk->k) tanh theta_j^{(kk,k)}
        //   O_{k,w_ij} = sum_kk B(kk->k) sigma^{(kk)}_i tanh theta_j^{(kk,k)}
        S *orow = A.O + s * P;
        for (int k = 0; k < K; k++) {
            S *ok = orow + size_t(k) * L;
            for (int p = tid; p < N + M; p += T) {
                S v = zero<S>();
                if (p < N) {
                    for (int kk = 0; kk < K; kk++) v = v + sm.bsig[(k * K + kk) * N + p];
                } else {
                    for (int kk = 0; kk < K; kk++) v = mad(sm.Bm[k * K + kk], sm.tnh[(kk * K + k) * M + p - N], v);
                }
                ok[p] = v;
            }
            // the w block with (i, j) stepped incrementally (no division per entry)
            S *ow = ok + N + M;
            int i = tid / M, j = tid - (tid / M) * M;
            const int di = T / M, dj = T - (T / M) * M;
            for (int p = tid; p < N * M; p += T) {
                S v = zero<S>();
                for (int kk = 0; kk < K; kk++) v = mad(sm.bsig[(k * K + kk) * N + i], sm.tnh[(kk * K + k) * M + j], v);
                ow[p] = v;
                j += dj;
                i += di;
                if (j >= M) {
                    j -= M;
                    i++;
                }
            }
        }
        __syncthreads();
    }
    if (writer && !A.cfg && A.accepted) A.accepted[c] = nacc;
}

// Evaluation at given configurations: where Phi (unscaled, phi) is rank
// deficient (e.g. two equal rows, whose amplitudes the sampler's threads may
// round differently), E = Phi^+ (D o Phi) with the Moore-Penrose
// pseudo-inverse, as the reference's completeOrthogonalDecomposition()
// .pseudoInverse() gives it (code/rbm.cc:1159-1171), and the configuration's
// O row is zero (det(Phi^+ Phi~) of a rank-deficient product). One thread per
// configuration; O rows are o_doubles doubles long.
__global__ void k_eval_singular(int count, int K, const cplx *phi, const cplx *dm, cplx *E, double *O,
                                size_t o_doubles) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= count) return;
    const int KK = K * K;
    cplx a[16], pinv[16], res[16];
    for (int t = 0; t < KK; t++) a[t] = phi[size_t(c) * KK + t];
    if (small_pinv(a, pinv, K) == K) return;
    for (int t = 0; t < KK; t++) res[t] = dm[size_t(c) * KK + t] * a[t];
    for (int r = 0; r < K; r++)
        for (int cc = 0; cc < K; cc++) {
            cplx e{0, 0};
            for (int t = 0; t < K; t++) e = e + pinv[r * K + t] * res[t * K + cc];
            E[size_t(c) * KK + r * K + cc] = e;
        }
    for (size_t t = 0; t < o_doubles; t++) O[size_t(c) * o_doubles + t] = 0.0;
}

// Per-step tables from the weights: cosh(2w), sinh(2w), exp(-2a), exp(2a).
template <class S>
__global__ void k_tables(Shape sh, const cplx *a, const cplx *w, S *ch, S *shh, S *eup, S *edn) {
    const size_t nw = size_t(sh.K) * sh.N * sh.M;
    for (size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x; t < nw; t += size_t(gridDim.x) * blockDim.x) {
        const S w2 = wt<S>(w[t]) * 2.0;
        ch[t] = ccosh_(w2);
        shh[t] = csinh_(w2);
        if (t < size_t(sh.K) * sh.N) {
            const S a2 = wt<S>(a[t]) * 2.0;
            eup[t] = cexp_(-a2);
            edn[t] = cexp_(a2);
        }
    }
}

}  // namespace

size_t sample_smem_bytes(const Shape &sh, int threads, bool complex_arith) {
    (void)threads;
    return smem_bytes(sh.N, sh.M, sh.K, complex_arith ? sizeof(cplx) : sizeof(double));
}

int sample_threads(int K, int tk) { return K * tk; }

// Raises the sampler's dynamic shared-memory limit; call outside stream capture.
template <class S, bool FILT, bool HEIS> cudaError_t prepare_variants() {
    cudaError_t e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample<S, 1, FILT, HEIS>));
    if (e == cudaSuccess)
        e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample<S, 2, FILT, HEIS>));
    if (e == cudaSuccess)
        e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample<S, 4, FILT, HEIS>));
    if (e == cudaSuccess)
        e = allow_max_dynamic_smem(reinterpret_cast<const void *>(k_sample<S, 8, FILT, HEIS>));
    return e;
}

template <class S> cudaError_t prepare_sample(const Shape &) {
    cudaError_t e = prepare_variants<S, false, false>();
    if (e == cudaSuccess) e = prepare_variants<S, false, true>();
    if constexpr (std::is_same<S, double>::value)
        if (e == cudaSuccess) e = prepare_variants<S, true, false>();
    return e;
}

template <class S, bool FILT, bool HEIS>
void launch_variant(const SampleArgs<S> &a, int U, int threads, size_t smem, cudaStream_t st) {
    if (U <= 1)
        k_sample<S, 1, FILT, HEIS><<<a.chains, threads, smem, st>>>(a);
    else if (U <= 2)
        k_sample<S, 2, FILT, HEIS><<<a.chains, threads, smem, st>>>(a);
    else if (U <= 4)
        k_sample<S, 4, FILT, HEIS><<<a.chains, threads, smem, st>>>(a);
    else
        k_sample<S, 8, FILT, HEIS><<<a.chains, threads, smem, st>>>(a);
}

// Launch with the smallest compiled units-per-thread bound that covers M/TK;
// the rejection filter runs when the FP32 tables are given (real arithmetic)
// and the local energy is ising-like (the Heisenberg-like form is its own
// instantiation, without the filter: the filter only skips work, its
// decisions are the unfiltered ones).
template <class S> cudaError_t launch_sample(const SampleArgs<S> &a, int threads, cudaStream_t st) {
    const size_t smem = smem_bytes(a.sh.N, a.sh.M, a.sh.K, sizeof(S));
    const int U = (a.sh.M + a.tk - 1) / a.tk;
    if (threads != sample_threads(a.sh.K, a.tk) || threads > kMaxThreads || U > kUMax || a.tk % 32)
        return cudaErrorInvalidConfiguration;
    bool filt = false;
    if constexpr (std::is_same<S, double>::value) filt = a.c32 && a.s32 && a.eu32 && a.ed32;
    if (a.ham) {
        launch_variant<S, false, true>(a, U, threads, smem, st);
    } else if (filt) {
        if constexpr (std::is_same<S, double>::value) launch_variant<S, true, false>(a, U, threads, smem, st);
    } else {
        launch_variant<S, false, false>(a, U, threads, smem, st);
    }
    return cudaGetLastError();
}

cudaError_t launch_eval_singular(int count, int K, const cplx *phi, const cplx *dm, cplx *E, double *O,
                                 size_t o_doubles, cudaStream_t st) {
    k_eval_singular<<<(count + 127) / 128, 128, 0, st>>>(count, K, phi, dm, E, O, o_doubles);
    return cudaGetLastError();
}

template cudaError_t prepare_sample<double>(const Shape &);
template cudaError_t prepare_sample<cplx>(const Shape &);

// out[e] = sum over chains of acc[chain][e], in chain order.
template <class S> __global__ void k_corr_reduce(const S *acc, int chains, size_t stride, S *out) {
    for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < stride; e += size_t(gridDim.x) * blockDim.x) {
        S s = zero<S>();
        for (int c = 0; c < chains; c++) s = s + acc[size_t(c) * stride + e];
        out[e] = s;
    }
}

template <class S> cudaError_t launch_corr_reduce(const S *acc, int chains, size_t stride, S *out, cudaStream_t st) {
    const int blocks = int(std::min<size_t>((stride + 255) / 256, 1024));
    k_corr_reduce<S><<<blocks, 256, 0, st>>>(acc, chains, stride, out);
    return cudaGetLastError();
}
template cudaError_t launch_corr_reduce<double>(const double *, int, size_t, double *, cudaStream_t);
template cudaError_t launch_corr_reduce<cplx>(const cplx *, int, size_t, cplx *, cudaStream_t);

template <class S>
cudaError_t launch_tables(const Shape &sh, const cplx *a, const cplx *w, S *ch, S *shh, S *eup, S *edn,
                          cudaStream_t st) {
    const size_t nw = size_t(sh.K) * sh.N * sh.M;
    int blocks = int(std::min<size_t>((nw + 255) / 256, 4096));
    k_tables<S><<<blocks, 256, 0, st>>>(sh, a, w, ch, shh, eup, edn);
    return cudaGetLastError();
}

template cudaError_t launch_sample<double>(const SampleArgs<double> &, int, cudaStream_t);
template cudaError_t launch_sample<cplx>(const SampleArgs<cplx> &, int, cudaStream_t);
template cudaError_t launch_tables<double>(const Shape &, const cplx *, const cplx *, double *, double *, double *,
                                           double *, cudaStream_t);
template cudaError_t launch_tables<cplx>(const Shape &, const cplx *, const cplx *, cplx *, cplx *, cplx *, cplx *,
                                         cudaStream_t);

}  // namespace nqes
