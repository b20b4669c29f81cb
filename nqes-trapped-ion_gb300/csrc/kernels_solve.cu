// Moments, matrix-free S·v and MINRES-QLP on the device.
//
// After sampling, the Ns × P log-derivative matrix O is resident in HBM
// (row s = sample, P = K·L contiguous). This file turns it into
//   * the moments of code/rbm.cc:640-650:
//       eloc = <E_loc>, o = <O>, skk = lambda (<|O|^2> - |o|^2),
//       f = <E_loc conj(O)> - eloc conj(o), e_mat = <E>;
//   * the S·v operator of code/rbm.cc:660-683:
//       (S v)_l = (1/Ns) sum_s conj(O_sl) (O_s · v) + skk_l v_l - (o · v) conj(o_l)
//     as two tall-skinny passes (u = O v, then y = O^H u);
//   * the MINRES-QLP iteration of code/minresqlp.h:158-389 (shift 0,
//     maxxnorm 1e7, Acondlim 1e15, TranCond 1e7, as called at
//     code/rbm.cc:661), with vectors on the device and the scalar recurrence
//     in a one-thread kernel, so that the whole solve runs inside one CUDA
//     graph (a conditional while node) without host round trips;
//   * the update w -= lr x of code/rbm.cc:699-717.
// All sums use a fixed order, so results are reproducible run to run.
#include <cmath>
#include <type_traits>

#include <utility>

#include "nqes_internal.h"

namespace nqes {
namespace {

constexpr int kVecThreads = 256;
// MINRES-QLP vector kernels: 64-thread blocks, so that at P = 4288 the 67
// blocks put one warp on each FP64 pipe they use (every FP64 warp
// instruction holds its pipe ~64 cycles) instead of two warps on 17 SMs.
constexpr int kMrThreads = 64;
__host__ __device__ constexpr int mr_blocks(int P) { return (P + kMrThreads - 1) / kMrThreads; }

__device__ __forceinline__ double ldg(const double *p) { return __ldg(p); }
__device__ __forceinline__ cplx ldg(const cplx *p) {
    double2 v = __ldg(reinterpret_cast<const double2 *>(p));
    return cplx{v.x, v.y};
}
template <class S> __device__ __forceinline__ double re_dot(S a, S b) { return re(a) * re(b) + im(a) * im(b); }

// Block sum of a double over the block's threads (a multiple of 32, fixed order).
__device__ double block_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (warp == 0) {
        r = lane < nw ? sh[lane] : 0.0;
        r = warp_sum(r);
    }
    __syncthreads();
    return r;  // valid in warp 0
}
template <class S> __device__ S block_sum_s(S v, double *sh);
template <> __device__ double block_sum_s<double>(double v, double *sh) { return block_sum(v, sh); }
template <> __device__ cplx block_sum_s<cplx>(cplx v, double *sh) {
    double r = block_sum(v.re, sh);
    double i = block_sum(v.im, sh);
    return cplx{r, i};
}
// Sum of n partials by one warp, strided then shuffled (fixed order).
__device__ __forceinline__ double warp_sum_array(const double *p, int n) {
    const int lane = threadIdx.x & 31;
    double s = 0.0;
    for (int t = lane; t < n; t += 32) s += p[t];
    return warp_sum(s);
}
template <class S> __device__ __forceinline__ S warp_sum_array_s(const S *p, int n) {
    const int lane = threadIdx.x & 31;
    S s = zero<S>();
    for (int t = lane; t < n; t += 32) s = s + p[t];
    return warp_sum(s);
}

// ---------------- moments ----------------

// e_mat = sum_s E_s / Ns and eloc = sum_s tr E_s / Ns (one block).
__global__ void k_emat(int Ns, int K, const cplx *E, cplx *emat, cplx *eloc) {
    __shared__ double sh[32];
    const int KK = K * K;
    for (int q = 0; q < KK; q++) {
        cplx acc{0, 0};
        for (int s = threadIdx.x; s < Ns; s += blockDim.x) acc += E[size_t(s) * KK + q];
        double r = block_sum(acc.re, sh), i = block_sum(acc.im, sh);
        if (threadIdx.x == 0) emat[q] = cplx{r / Ns, i / Ns};
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        cplx t{0, 0};
        for (int k = 0; k < K; k++) t += emat[k * K + k];
        // mean of the traces = eloc / Ns of code/rbm.cc:640
        eloc[0] = t;
    }
}

// Partial column sums over a chunk of rows: o, |O|^2 and E_loc conj(O).
// Launched with kVecThreads threads: the block stages the local energies
// (traces of E) of kVecThreads samples at a time in shared memory, so a column
// costs three FP64 operations per sample.
template <class S, class TO>
__global__ void __launch_bounds__(kVecThreads) k_moment_part(int Ns, int P, int K, int rchunks, const TO *O,
                                                             const cplx *E, S *po, double *ps2, S *pf) {
    __shared__ S els[kVecThreads];
    const int p = blockIdx.x * kVecThreads + threadIdx.x;
    const int r = blockIdx.y;
    const int s0 = int(int64_t(Ns) * r / rchunks), s1 = int(int64_t(Ns) * (r + 1) / rchunks);
    const int KK = K * K;
    S o = zero<S>(), f = zero<S>();
    double s2 = 0.0;
    for (int t0 = s0; t0 < s1; t0 += kVecThreads) {
        const int nt = min(kVecThreads, s1 - t0);
        if (int(threadIdx.x) < nt) {
            const size_t s = size_t(t0) + threadIdx.x;
            cplx el{0, 0};
            for (int k = 0; k < K; k++) el += E[s * KK + k * K + k];
            els[threadIdx.x] = from_c<S>(el);
        }
        __syncthreads();
        if (p < P) {
            const TO *col = O + size_t(t0) * P + p;
            for (int q = 0; q < nt; q++) {
                const S v = col[size_t(q) * P];
                o = o + v;
                s2 += norm2(v);
                f = cmad(v, els[q], f);  // conj(O) * E_loc
            }
        }
        __syncthreads();
    }
    if (p >= P) return;
    po[size_t(r) * P + p] = o;
    ps2[size_t(r) * P + p] = s2;
    pf[size_t(r) * P + p] = f;
}

// The same partial column sums over O stored as double-float pairs (hi, lo)
// in its FP64 slots (real arithmetic): o, |O|^2 and E_loc O accumulated in
// double-float on the FP32 pipe (products with their FMA error terms, sums
// TwoSum-compensated: a few 2^-48 of the sums of |terms|), converted to FP64
// once per partial.
__global__ void __launch_bounds__(kVecThreads) k_moment_part_split(int Ns, int P, int K, int rchunks, const float2 *O,
                                                                   const cplx *E, double *po, double *ps2, double *pf) {
    __shared__ float2 els[kVecThreads];
    const int p = blockIdx.x * kVecThreads + threadIdx.x;
    const int r = blockIdx.y;
    const int s0 = int(int64_t(Ns) * r / rchunks), s1 = int(int64_t(Ns) * (r + 1) / rchunks);
    const int KK = K * K;
    float oh = 0.f, ol = 0.f, qh = 0.f, ql = 0.f, fh = 0.f, fl = 0.f;
    for (int t0 = s0; t0 < s1; t0 += kVecThreads) {
        const int nt = min(kVecThreads, s1 - t0);
        if (int(threadIdx.x) < nt) {
            const size_t s = size_t(t0) + threadIdx.x;
            double el = 0.0;
            for (int k = 0; k < K; k++) el += E[s * KK + k * K + k].re;
            float eh, elo;
            df_split(el, eh, elo);
            els[threadIdx.x] = make_float2(eh, elo);
        }
        __syncthreads();
        if (p < P) {
            const float2 *col = O + size_t(t0) * P + p;
            for (int q = 0; q < nt; q++) {
                const float2 v = col[size_t(q) * P];
                const float2 e = els[q];
                df_acc(oh, ol, v.x, v.y);
                df_fma(qh, ql, v.x, v.y, v.x, v.y);
                df_fma(fh, fl, v.x, v.y, e.x, e.y);  // real: conj(O) E = O E
            }
        }
        __syncthreads();
    }
    if (p >= P) return;
    po[size_t(r) * P + p] = double(oh) + double(ol);
    ps2[size_t(r) * P + p] = double(qh) + double(ql);
    pf[size_t(r) * P + p] = double(fh) + double(fl);
}

template <class S>
__global__ void k_moment_final(int Ns, int P, int rchunks, const StepParams *sp, const S *po, const double *ps2,
                               const S *pf, const cplx *eloc, S *o, S *skk, S *f, int *err) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    S so = zero<S>(), sf = zero<S>();
    double s2 = 0.0;
    for (int r = 0; r < rchunks; r++) {
        so = so + po[size_t(r) * P + p];
        s2 += ps2[size_t(r) * P + p];
        sf = sf + pf[size_t(r) * P + p];
    }
    const double inv_ns = 1.0 / double(Ns);
    const S el = from_c<S>(eloc[0]);  // mean local energy
    const S om = so * inv_ns;
    const double dg = (s2 * inv_ns - norm2(om)) * sp->reglam;
    // f = <E conj(O)> - eloc conj(o)
    const S fv = sf * inv_ns - el * conj(om);
    o[p] = om;
    skk[p] = one<S>() * dg;
    f[p] = fv;
    if (!finite(om) || !isfinite(dg) || !finite(fv)) atomicOr(err, kErrNonFinite);
}

// ---------------- S·v ----------------

// u_s = sum_p O_sp v_p: one warp per row.
template <class S> __global__ void k_sv_rows(int Ns, int P, const S *O, const S *v, S *u, const int *guard) {
    if (loop_guard_off(guard)) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= Ns) return;
    const S *row = O + size_t(warp) * P;
    S acc = zero<S>();
    for (int p = lane; p < P; p += 32) acc = mad(row[p], ldg(v + p), acc);
    acc = warp_sum(acc);
    if (lane == 0) u[warp] = acc;
}

// ypart[r][p] = sum_{s in chunk r} conj(O_sp) u_s
template <class S>
__global__ void k_sv_cols(int Ns, int P, int rchunks, const S *O, const S *u, S *ypart, const int *guard) {
    if (loop_guard_off(guard)) return;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    if (p >= P) return;
    const int s0 = int(int64_t(Ns) * r / rchunks), s1 = int(int64_t(Ns) * (r + 1) / rchunks);
    S acc = zero<S>();
    for (int s = s0; s < s1; s++) acc = cmad(O[size_t(s) * P + p], ldg(u + s), acc);
    ypart[size_t(r) * P + p] = acc;
}

__global__ void k_to_f32(int n, const double *x, float *y) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) y[t] = float(x[t]);
}

__device__ __forceinline__ void mirror_f32(float *v32, int p, double v) {
    if (v32) v32[p] = float(v);
}
__device__ __forceinline__ void mirror_f32(float *, int, cplx) {}

// S·v epilogue for column p. The column sums of the row-chunk partials are
// split over kRG groups of threads per column so that many loads are in flight
// (one thread walking ~150 partials is load-latency bound); the groups then
// combine in a fixed order.
constexpr int kRG = 8;
constexpr int kMrColThreads = kMrThreads * kRG;

// hi + lo += x exactly (TwoSum): a two-float accumulator on the FP32 pipe.
__device__ __forceinline__ void two_sum_acc(float &hi, float &lo, float x) {
    const float sum = hi + x, bb = sum - hi;
    lo += (hi - (sum - bb)) + (x - bb);
    hi = sum;
}

template <class S> struct ColSumSmem {
    float hi[kRG][kMrThreads], lo[kRG][kMrThreads];
    S y[kRG][kMrThreads];
};

// sum over r of ypart[r][p] in the threads of group 0 (pl = column in the block,
// rg = group); every thread of the block must call it. FP32 partials (mixed
// form) are summed with two-float accumulators, converted to FP64 once.
template <class S>
__device__ S sv_colsum(const SolveBufs<S> &B, int p, int pl, int rg, ColSumSmem<S> &cs) {
    const int R = B.fact ? B.rchunks : B.svp, r0 = int(int64_t(R) * rg / kRG), r1 = int(int64_t(R) * (rg + 1) / kRG);
    const bool in = p < B.sh.P;
    S y = zero<S>();
    if (B.fact) {
        float hi = 0.f, lo = 0.f;
        if (in)
            for (int r = r0; r < r1; r++) two_sum_acc(hi, lo, B.ypart32[size_t(r) * B.sh.P + p]);
        cs.hi[rg][pl] = hi;
        cs.lo[rg][pl] = lo;
        __syncthreads();
        if (rg == 0) {
            hi = cs.hi[0][pl];
            lo = cs.lo[0][pl];
            for (int g = 1; g < kRG; g++) {
                two_sum_acc(hi, lo, cs.hi[g][pl]);
                lo += cs.lo[g][pl];
            }
            y = one<S>() * (double(hi) + double(lo));
        }
    } else {
        if (in)
            for (int r = r0; r < r1; r++) y = y + B.ysv[size_t(r) * B.sh.P + p];
        cs.y[rg][pl] = y;
        __syncthreads();
        if (rg == 0) {
            y = cs.y[0][pl];
            for (int g = 1; g < kRG; g++) y = y + cs.y[g][pl];
        }
    }
    return y;
}

// out = column sum / Ns + skk v - (o·v) conj(o) (code/rbm.cc:660-683).
template <class S>
__device__ __forceinline__ S sv_finish(const SolveBufs<S> &B, int p, const S *v, S ov, S y) {
    y = y * (1.0 / double(B.Ns));
    y = mad(B.skk[p], v[p], y);
    y = y - ov * conj(B.o[p]);
    return y;
}

template <class S> __global__ void __launch_bounds__(kMrColThreads) k_apply_out(SolveBufs<S> B, const S *v, S *out) {
    __shared__ S ovs;
    __shared__ ColSumSmem<S> cs;
    if (threadIdx.x < 32) {
        S ov = warp_sum_array_s(B.ovpart, mr_blocks(B.sh.P));
        if (threadIdx.x == 0) ovs = ov;
    }
    const int pl = threadIdx.x % kMrThreads, rg = threadIdx.x / kMrThreads;
    const int p = blockIdx.x * kMrThreads + pl;
    const S y = sv_colsum(B, p, pl, rg, cs);  // its barrier also publishes ovs
    if (rg == 0 && p < B.sh.P) out[p] = sv_finish(B, p, v, ovs, y);
}

// Per-block partials of o·v (no conjugation, code/rbm.cc:673-676).
template <class S> __global__ void k_ov_part(int P, const S *o, const S *v, S *ovpart) {
    __shared__ double sh[32];
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    S t = p < P ? o[p] * v[p] : zero<S>();
    S s = block_sum_s(t, sh);
    if (threadIdx.x == 0) ovpart[blockIdx.x] = s;
}

// ---------------- MINRES-QLP ----------------

constexpr int kInternal = -2, kEigvec = -1, kZero = 0, kConv = 1, kConvLS = 2, kEps1 = 3, kEpsLS = 4,
              kEigConv = 5, kXNorm = 6, kACond = 7, kMaxIt = 8, kSingular = 9;
constexpr double kMaxXNorm = 1e7, kACondLim = 1e15, kTranCond = 1e7;

// r1 = r2 = r3 = b, x = w = wl = wl2 = xl2 = 0, v = b / beta1, o·v partials.
template <class S> __global__ void k_minres_init_vec(SolveBufs<S> B) {
    __shared__ double sh[32];
    const int P = B.sh.P, p = blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0;
    if (p < P) {
        const S b = B.f[p];
        t = norm2(b);
        B.r1[p] = b;
        B.r2[p] = b;
        B.r3[p] = b;
        B.x[p] = zero<S>();
        B.w[p] = zero<S>();
        B.wl[p] = zero<S>();
        B.wl2[p] = zero<S>();
        B.xl2[p] = zero<S>();
    }
    t = block_sum(t, sh);
    if (threadIdx.x == 0) B.part[2 * kPartStride + blockIdx.x] = t;
}

template <class S> __global__ void k_minres_init_scalar(SolveBufs<S> B) {
    QlpState &q = *B.qs;
    const int nb = mr_blocks(B.sh.P);
    const double b2 = warp_sum_array(B.part + 2 * kPartStride, nb);
    if (threadIdx.x != 0) return;
    const double beta1 = sqrt(b2);
    q = QlpState{};
    q.beta1 = beta1;
    q.phi = beta1;
    q.betan = beta1;
    q.cs = -1; q.cr1 = -1; q.cr2 = -1;
    q.rnorm = beta1;
    q.acond = 1;
    q.relres = beta1 / (beta1 + 1e-50);
    q.flag = beta1 == 0 ? kZero : kInternal;
    const unsigned long long mi = B.sp->maxit;
    q.cap = mi;
    q.running = (q.flag == kInternal && mi > 0) ? 1 : 0;
    LzState &lz = *B.lz;
    lz.j = 1;
    lz.beta[0] = 0;
    lz.beta[1] = beta1;
    lz.beta[2] = 0;
    lz.arrived = 0;
    if (!isfinite(beta1)) {
        atomicOr(B.err, kErrMinresNonFinite);
        q.running = 0;
    }
}

// v = r3 / beta (first iteration) and o·v partials.
template <class S> __global__ void k_minres_first_v(SolveBufs<S> B) {
    __shared__ double sh[32];
    const int P = B.sh.P, p = blockIdx.x * blockDim.x + threadIdx.x;
    const double beta = B.qs->betan;
    S t = zero<S>();
    if (p < P) {
        const S v = B.r3[p] * (1.0 / beta);
        B.v[p] = v;
        B.vq[size_t(1) * P + p] = v;
        mirror_f32(B.v32, p, v);
        t = B.o[p] * v;
    }
    S s = block_sum_s(t, sh);
    if (threadIdx.x == 0) B.ovpart[blockIdx.x] = s;
}

// Lanczos part 1 of step j: r3 = S v_j - (beta_j / beta_{j-1}) r1; partials
// of Re(r3^H v_j). The Lanczos chain runs whether or not the QLP chain beside
// it ends the solve (a step past the end only costs its time).
template <class S> __device__ __forceinline__ void lanczos_a_body(const SolveBufs<S> &B, const int bid) {
    __shared__ double sh[32];
    __shared__ S ovs;
    __shared__ ColSumSmem<S> cs;
    if (loop_guard_off(B.guard)) return;
    const LzState &lz = *B.lz;
    const unsigned long long j = lz.j;
    const int nb = mr_blocks(B.sh.P);
    if (threadIdx.x < 32) {
        S ov = warp_sum_array_s(B.ovpart, nb);
        if (threadIdx.x == 0) ovs = ov;
    }
    const int P = B.sh.P, pl = threadIdx.x % kMrThreads, rg = threadIdx.x / kMrThreads;
    const int p = bid * kMrThreads + pl;
    const S y = sv_colsum(B, p, pl, rg, cs);  // its barrier also publishes ovs
    const bool first = j == 1;
    const double c1 = first ? 0.0 : lz.beta[j % 3] / lz.beta[(j - 1) % 3];  // beta_new / betal_new
    double t = 0.0;
    if (rg == 0 && p < P) {
        S r3 = sv_finish(B, p, B.v, ovs, y);
        if (!first) r3 = r3 - B.r1[p] * c1;
        B.r3[p] = r3;
        t = re_dot(r3, B.v[p]);
    }
    t = block_sum(t, sh);
    if (threadIdx.x == 0) B.part[bid] = t;
}
// Programmatic dependent launch: the loop body's kernels after the first on
// each stream are launched with programmatic stream serialisation, so that
// a kernel is scheduled while its predecessor drains; it waits here for the
// predecessor's completion and memory before reading anything (a no-op when
// launched without the attribute).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <class S> __global__ void __launch_bounds__(kMrColThreads) k_lanczos_a(SolveBufs<S> B) {
    pdl_wait();
    lanczos_a_body(B, blockIdx.x);
}

// Lanczos part 2 of step j: r3 -= (alfa_j / beta_j) r2; r1 = r2; r2 = r3;
// partials of |r3|^2.
template <class S> __device__ __forceinline__ void lanczos_b_body(const SolveBufs<S> &B, const int bid) {
    __shared__ double sh[32];
    __shared__ double alfa_s;
    if (loop_guard_off(B.guard)) return;
    const LzState &lz = *B.lz;
    const unsigned long long j = lz.j;
    const int nb = mr_blocks(B.sh.P);
    if (threadIdx.x < 32) {
        double a = warp_sum_array(B.part, nb);
        if (threadIdx.x == 0) alfa_s = a;
    }
    __syncthreads();
    const int P = B.sh.P, p = bid * blockDim.x + threadIdx.x;
    const double c2 = alfa_s / lz.beta[j % 3];  // alfa / beta_new
    double t = 0.0;
    if (p < P) {
        S r3 = B.r3[p] - B.r2[p] * c2;
        B.r1[p] = B.r2[p];
        B.r2[p] = r3;
        B.r3[p] = r3;
        t = norm2(r3);
    }
    t = block_sum(t, sh);
    if (threadIdx.x == 0) B.part[kPartStride + bid] = t;
}
template <class S> __global__ void k_lanczos_b(SolveBufs<S> B) {
    pdl_wait();
    lanczos_b_body(B, blockIdx.x);
}

// Lanczos part 3 of step j: beta_{j+1} = |r3|, v_{j+1} = r3 / beta_{j+1} (into
// v, its FP32 mirror and the QLP chain's slot), o·v_{j+1} partials; the last
// block to finish publishes alfa_j, |r3_j|^2 and beta_{j+1} and advances j
// (every block read j before any block arrived).
template <class S> __device__ __forceinline__ void lanczos_next_body(const SolveBufs<S> &B, const int bid) {
    __shared__ double sh[32];
    __shared__ double s_alfa, s_bn2;
    __shared__ int last;
    if (loop_guard_off(B.guard)) return;
    LzState &lz = *B.lz;
    const unsigned long long j = lz.j;
    const int nb = mr_blocks(B.sh.P);
    if (threadIdx.x < 32) {
        const double a = warp_sum_array(B.part, nb);
        const double b2 = warp_sum_array(B.part + kPartStride, nb);
        if (threadIdx.x == 0) {
            s_alfa = a;
            s_bn2 = b2;
        }
    }
    __syncthreads();
    const double betan = sqrt(s_bn2);
    const int P = B.sh.P, p = bid * blockDim.x + threadIdx.x;
    S *vq = B.vq + size_t((j + 1) % 3) * P;
    S ovt = zero<S>();
    if (p < P) {
        const S vn = B.r3[p] * (1.0 / betan);
        B.v[p] = vn;
        vq[p] = vn;
        mirror_f32(B.v32, p, vn);
        ovt = B.o[p] * vn;
    }
    S s = block_sum_s(ovt, sh);
    if (threadIdx.x == 0) {
        B.ovpart[bid] = s;
        __threadfence();
        last = atomicAdd(&lz.arrived, 1u) == unsigned(nb) - 1;  // nb blocks per solve
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        lz.alfa[j & 1] = s_alfa;
        lz.bn2[j & 1] = s_bn2;
        lz.beta[(j + 1) % 3] = betan;
        lz.arrived = 0;
        lz.j = j + 1;
        __threadfence();
    }
}
template <class S> __global__ void k_lanczos_next(SolveBufs<S> B) {
    pdl_wait();
    lanczos_next_body(B, blockIdx.x);
}

__device__ __forceinline__ double sgn(double a) { return copysign(1.0, a); }
__device__ void givens(double a, double b, double &c, double &s, double &r) {
    if (b == 0) {
        c = (a == 0) ? 1.0 : sgn(a);
        s = 0;
        r = fabs(a);
    } else if (a == 0) {
        c = 0;
        s = sgn(b);
        r = fabs(b);
    } else if (fabs(b) > fabs(a)) {
        const double t = a / b;
        s = sgn(b) / sqrt(1 + t * t);
        c = s * t;
        r = b / s;
    } else {
        const double t = b / a;
        c = sgn(a) / sqrt(1 + t * t);
        s = c * t;
        r = a / c;
    }
}

// The scalar part of one MINRES-QLP iteration (code/minresqlp.h:158-374), in
// the reference's order, recording the coefficients the vector kernel needs.
// q is a register copy of the state: every FP64 instruction of this one-thread
// chain costs ~64 cycles, so none of them waits on a global load in between.
template <class S>
__device__ __forceinline__ void qlp_scalar_step(const SolveBufs<S> &B, QlpState &q, double alfa, double bn2) {
    q.iters++;
    const double betal = q.beta;
    q.beta = q.betan;
    q.alfa = alfa;
    q.betan = sqrt(bn2);
    const unsigned long long iters = q.iters;
    q.mode = 0;
    q.qlp_first = 0;
    if (!isfinite(alfa) || !isfinite(q.betan)) {
        atomicOr(B.err, kErrMinresNonFinite);
        q.running = 0;
        if (B.use_cond) cudaGraphSetConditional(B.cond, 0);
        return;
    }
    if (iters == 1 && q.betan == 0) {
        if (alfa == 0) {
            q.flag = kZero;
        } else {
            q.flag = kEigvec;
            q.mode = 3;  // x = b / alfa
        }
        q.running = 0;
        if (B.use_cond) cudaGraphSetConditional(B.cond, 0);
        return;
    }
    const double betan = q.betan;
    const double pnorm = sqrt(betal * betal + alfa * alfa + betan * betan);

    // previous left rotation Q_{k-1}
    const double dbar = q.dltan;
    double dlta = q.cs * dbar + q.sn * alfa;
    const double epln = q.eplnn;
    const double gbar = q.sn * dbar - q.cs * alfa;
    q.eplnn = q.sn * betan;
    q.dltan = -q.cs * betan;
    const double dlta_qlp = dlta;
    // current left rotation Q_k
    const double gamal3 = q.gamal2;
    q.gamal2 = q.gamal;
    q.gamal = q.gama;
    givens(gbar, betan, q.cs, q.sn, q.gama);
    const double gama_tmp = q.gama;
    const double taul2 = q.taul;
    q.taul = q.tau;
    q.tau = q.cs * q.phi;
    q.axnorm = sqrt(q.axnorm * q.axnorm + q.tau * q.tau);
    q.phi = q.sn * q.phi;
    // previous right rotation P_{k-2,k}
    if (iters > 2) {
        q.veplnl2 = q.veplnl;
        q.etal2 = q.etal;
        q.etal = q.eta;
        const double dlta_tmp = q.sr2 * q.vepln - q.cr2 * dlta;
        q.veplnl = q.cr2 * q.vepln + q.sr2 * dlta;
        dlta = dlta_tmp;
        q.eta = q.sr2 * q.gama;
        q.gama = -q.cr2 * q.gama;
    }
    // current right rotation P_{k-1,k}
    if (iters > 1) {
        givens(q.gamal, dlta, q.cr1, q.sr1, q.gamal);
        q.vepln = q.sr1 * q.gama;
        q.gama = -q.cr1 * q.gama;
    }
    // solution norm
    const double ul4 = q.ul3;
    q.ul3 = q.ul2;
    if (iters > 2) q.ul2 = (taul2 - q.etal2 * ul4 - q.veplnl2 * q.ul3) / q.gamal2;
    if (iters > 1) q.ul = (q.taul - q.etal * q.ul3 - q.veplnl * q.ul2) / q.gamal;
    const double xnorm_tmp = sqrt(q.xl2norm * q.xl2norm + q.ul2 * q.ul2 + q.ul * q.ul);
    if (fabs(q.gama) > 2.2250738585072014e-308 && xnorm_tmp < kMaxXNorm) {
        q.u = (q.tau - q.eta * q.ul2 - q.vepln * q.ul) / q.gama;
        if (sqrt(xnorm_tmp * xnorm_tmp + q.u * q.u) > kMaxXNorm) {
            q.u = 0;
            q.flag = kXNorm;
        }
    } else {
        q.u = 0;
        q.flag = kSingular;
    }
    q.xl2norm = sqrt(q.xl2norm * q.xl2norm + q.ul2 * q.ul2);
    q.xnorm = sqrt(q.xl2norm * q.xl2norm + q.ul * q.ul + q.u * q.u);

    // choose the w / x update (applied by k_qlp_vectors)
    if (q.acond < kTranCond && q.flag != kInternal && q.qlp_iters == 0) {
        q.mode = (q.xnorm < kMaxXNorm) ? 1 : 4;  // 4: MINRES w update without x
        if (q.mode == 4) q.flag = kXNorm;
        q.epln = epln;
        q.dlta_qlp = dlta_qlp;
        q.gama_tmp = gama_tmp;
    } else {
        q.qlp_iters++;
        q.mode = 2;
        q.qlp_first = (q.qlp_iters == 1 && iters > 1) ? 1 : 0;
        q.gamal3 = gamal3;
        q.veplnl2_v = q.veplnl2;
        q.etal_v = q.etal;
        q.w_gamal_qlp = q.gamal_qlp;
        q.w_vepln_qlp = q.vepln_qlp;
        q.w_gama_qlp = q.gama_qlp;
        q.w_ul_qlp = q.ul_qlp;
        q.w_u_qlp = q.u_qlp;
    }
    q.iters_snapshot = iters;
    q.cr2_v = q.cr2;
    q.sr2_v = q.sr2;

    // next right rotation P_{k-1,k+1}
    const double gamal_tmp = q.gamal;
    givens(q.gamal, q.eplnn, q.cr2, q.sr2, q.gamal);
    q.gamal_qlp = gamal_tmp;
    q.vepln_qlp = q.vepln;
    q.gama_qlp = q.gama;
    q.ul_qlp = q.ul;
    q.u_qlp = q.u;
    // norm and condition estimates
    const double abs_gama = fabs(q.gama);
    q.anorm = fmax(fmax(q.anorm, pnorm), fmax(q.gamal, abs_gama));
    if (iters == 1) {
        q.gmin = q.gama;
        q.gminl = q.gmin;
    } else {
        const double gminl2 = q.gminl;
        q.gminl = q.gmin;
        q.gmin = fmin(fmin(gminl2, q.gamal), abs_gama);
    }
    const double acondl = q.acond;
    q.acond = q.anorm / q.gmin;
    const double rnorml = q.rnorm;
    const double relresl = q.relres;
    if (q.flag != kSingular) q.rnorm = q.phi;
    q.relres = q.rnorm / (q.anorm * q.xnorm + q.beta1);
    const double rootl = sqrt(gbar * gbar + q.dltan * q.dltan);
    const double relaresl = rootl / q.anorm;
    const double epsx = q.anorm * q.xnorm * 2.220446049250313e-16;
    if (q.flag == kInternal || q.flag == kSingular) {
        const double t1 = 1 + q.relres, t2 = 1 + relaresl;
        if (iters >= q.cap) q.flag = kMaxIt;
        if (q.acond >= kACondLim) q.flag = kACond;
        if (q.xnorm >= kMaxXNorm) q.flag = kXNorm;
        if (epsx >= q.beta1) q.flag = kEigConv;
        if (t2 <= 1) q.flag = kEpsLS;
        if (t1 <= 1) q.flag = kEps1;
        if (relaresl <= B.sp->rtol) q.flag = kConvLS;
        if (q.relres <= B.sp->rtol) q.flag = kConv;
    }
    if (q.flag == kConvLS || q.flag == kEpsLS || q.flag == kXNorm || q.flag == kACond) {
        q.iters--;
        q.acond = acondl;
        q.rnorm = rnorml;
        q.relres = relresl;
    }
    if (!isfinite(q.relres) || !isfinite(q.anorm) || !isfinite(q.xnorm) || !isfinite(q.gama)) {
        atomicOr(B.err, kErrMinresNonFinite);
        q.flag = kInternal;
        q.running = 0;
        if (B.use_cond) cudaGraphSetConditional(B.cond, 0);
        return;
    }
    q.running = (q.flag == kInternal && q.iters < q.cap) ? 1 : 0;
    if (B.use_cond) cudaGraphSetConditional(B.cond, q.running);
}

template <class S> __device__ __forceinline__ void qlp_scalar_body(const SolveBufs<S> &B) {
    QlpState &gq = *B.qs;
    if (threadIdx.x == 0) gq.bodies++;
    if (!gq.running) {
        // The while node's condition defaults to 1 on every graph launch; a
        // solve that needs no iteration (b = 0, maxit = 0) ends the loop here.
        gq.mode = 0;
        if (B.use_cond && threadIdx.x == 0) cudaGraphSetConditional(B.cond, 0);
        return;
    }
    if (threadIdx.x != 0) return;
    QlpState q = gq;
    // alfa_j and |r3_j|^2 of this step, published by the Lanczos chain
    const LzState &lz = *B.lz;
    const unsigned long long j = q.iters + 1;
    const double alfa = lz.alfa[j & 1], bn2 = lz.bn2[j & 1];
    qlp_scalar_step(B, q, alfa, bn2);
    gq = q;
}
template <class S> __global__ void k_qlp_scalar(SolveBufs<S> B) { qlp_scalar_body(B); }

// Vector part: w / x updates (code/minresqlp.h:253-299) with v_j from the
// QLP chain's slot.
template <class S> __device__ __forceinline__ void qlp_vectors_body(const SolveBufs<S> &B, const int bid) {
    const QlpState &q = *B.qs;
    const int P = B.sh.P, p = bid * blockDim.x + threadIdx.x;
    if (q.mode == 0 && !q.running) return;
    if (p < P) {
        const S v = B.vq[size_t(q.iters_snapshot % 3) * P + p];
        S w = B.w[p], wl = B.wl[p], wl2 = B.wl2[p], x = B.x[p], xl2 = B.xl2[p];
        const unsigned long long it = q.iters_snapshot;
        if (q.mode == 1 || q.mode == 4) {
            wl2 = wl;
            wl = w;
            w = (v - wl2 * q.epln - wl * q.dlta_qlp) * (1.0 / q.gama_tmp);
            if (q.mode == 1) x = mad(one<S>() * q.tau, w, x);
        } else if (q.mode == 2) {
            if (q.qlp_first) {
                if (it > 3) wl2 = wl2 * q.gamal3 + wl * q.veplnl2_v + w * q.etal_v;
                if (it > 2) wl = wl * q.w_gamal_qlp + w * q.w_vepln_qlp;
                w = w * q.w_gama_qlp;
                xl2 = x - wl * q.w_ul_qlp - w * q.w_u_qlp;
            }
            if (it == 1) {
                wl2 = wl;
                wl = v * q.sr1;
                w = -(v * q.cr1);
            } else if (it == 2) {
                wl2 = wl;
                const S w0 = w;
                wl = w0 * q.cr1 + v * q.sr1;
                w = w0 * q.sr1 - v * q.cr1;
            } else {
                const S p_wl = wl, p_w = w;
                const S nw = p_wl * q.sr2_v - v * q.cr2_v;
                const S nwl2 = p_wl * q.cr2_v + v * q.sr2_v;
                const S t = p_w * q.cr1 + nw * q.sr1;
                w = p_w * q.sr1 - nw * q.cr1;
                wl = t;
                wl2 = nwl2;
            }
            xl2 = xl2 + wl2 * q.ul2;
            x = xl2 + wl * q.ul + w * q.u;
        } else if (q.mode == 3) {
            x = B.f[p] * (1.0 / q.alfa);
        }
        B.w[p] = w;
        B.wl[p] = wl;
        B.wl2[p] = wl2;
        B.x[p] = x;
        B.xl2[p] = xl2;
    }
}
template <class S> __global__ void k_qlp_vectors(SolveBufs<S> B) {
    pdl_wait();
    qlp_vectors_body(B, blockIdx.x);
}

// w -= lr x in the reference layout (code/rbm.cc:699-717).
template <class S>
__global__ void k_update(Shape sh, const StepParams *sp, const S *x, cplx *a, cplx *b, cplx *w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= sh.P) return;
    const int k = t / sh.L, p = t - k * sh.L;
    const cplx d = to_c(x[t]) * sp->lr;
    if (p < sh.N) {
        a[k * sh.N + p] -= d;
    } else if (p < sh.N + sh.M) {
        b[k * sh.M + (p - sh.N)] -= d;
    } else {
        const int q = p - sh.N - sh.M;
        w[size_t(k) * sh.N * sh.M + q] -= d;
    }
}

// The batched MINRES-QLP loop runs while any member's solve runs.
__global__ void k_batch_cond(const int *const *flags, int n, cudaGraphConditionalHandle cond) {
    int any = 0;
    for (int i = threadIdx.x; i < n; i += 32) any |= *reinterpret_cast<const volatile int *>(flags[i]) != 0;
    any = __any_sync(0xffffffffu, any);
    if (threadIdx.x == 0) cudaGraphSetConditional(cond, any ? 1u : 0u);
}

// ---- grouped launches (the loop body of a batch) ----
// One launch runs the same kernel for every solve of a group: block b belongs
// to solve m with first[m] <= b < first[m + 1] and runs as that solve's block
// b - first[m] with the solve's own buffers, so every solve does exactly the
// arithmetic of its own launch, in the same order.
template <class S>
__global__ void __launch_bounds__(kMrColThreads)
    k_lanczos_a_g(const SolveBufs<S> *__restrict__ tab, const int *__restrict__ first, int n) {
    const int m = group_member(first, n, blockIdx.x);
    lanczos_a_body(tab[m], int(blockIdx.x) - __ldg(first + m));
}
template <class S>
__global__ void k_lanczos_b_g(const SolveBufs<S> *__restrict__ tab, const int *__restrict__ first, int n) {
    const int m = group_member(first, n, blockIdx.x);
    lanczos_b_body(tab[m], int(blockIdx.x) - __ldg(first + m));
}
template <class S>
__global__ void k_lanczos_next_g(const SolveBufs<S> *__restrict__ tab, const int *__restrict__ first, int n) {
    const int m = group_member(first, n, blockIdx.x);
    lanczos_next_body(tab[m], int(blockIdx.x) - __ldg(first + m));
}
template <class S> __global__ void k_qlp_scalar_g(const SolveBufs<S> *__restrict__ tab) { qlp_scalar_body(tab[blockIdx.x]); }
template <class S>
__global__ void k_qlp_vectors_g(const SolveBufs<S> *__restrict__ tab, const int *__restrict__ first, int n) {
    const int m = group_member(first, n, blockIdx.x);
    qlp_vectors_body(tab[m], int(blockIdx.x) - __ldg(first + m));
}

}  // namespace

int minres_vector_blocks(int P) { return mr_blocks(P); }

template <class S>
cudaError_t launch_lanczos_group(const SolveBufs<S> *tab, const int *first, int n, int blocks, cudaStream_t st) {
    k_lanczos_a_g<S><<<blocks, kMrColThreads, 0, st>>>(tab, first, n);
    k_lanczos_b_g<S><<<blocks, kMrThreads, 0, st>>>(tab, first, n);
    k_lanczos_next_g<S><<<blocks, kMrThreads, 0, st>>>(tab, first, n);
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_qlp_group(const SolveBufs<S> *tab, const int *first, int n, int blocks, cudaStream_t st) {
    k_qlp_scalar_g<S><<<n, 32, 0, st>>>(tab);
    k_qlp_vectors_g<S><<<blocks, kMrThreads, 0, st>>>(tab, first, n);
    return cudaGetLastError();
}

cudaError_t launch_batch_cond(const int *const *flags, int n, cudaGraphConditionalHandle cond, cudaStream_t st) {
    k_batch_cond<<<1, 32, 0, st>>>(flags, n, cond);
    return cudaGetLastError();
}

template <class S> cudaError_t launch_moments(const SolveBufs<S> &B, cudaStream_t st) {
    const int P = B.sh.P, nb = (P + kVecThreads - 1) / kVecThreads;
    k_emat<<<1, 1024, 0, st>>>(B.Ns, B.sh.K, B.E, B.emat, B.eloc);
    // partial buffers reuse the ypart region (rchunks × P of S) and the r1/r2 vectors
    S *po = B.ypart;
    S *pf = B.ypart + size_t(B.rchunks) * P;
    double *ps2 = reinterpret_cast<double *>(B.ypart + size_t(2) * B.rchunks * P);
    dim3 g(nb, B.rchunks);
    if constexpr (std::is_same<S, double>::value) {
        if (B.fact) {
            float *fo = B.ypart32, *ff = fo + size_t(B.rchunks) * P, *fs = ff + size_t(B.rchunks) * P;
            cudaError_t e = launch_fmoments(B.F, B.E, fo, ff, fs, st);
            if (e == cudaSuccess)
                e = launch_fmoment_final(B.F, B.sp, fo, ff, fs, B.eloc, B.o, B.skk, B.f, B.err, st);
            return e;
        }
        if (B.o_split) {
            k_moment_part_split<<<g, kVecThreads, 0, st>>>(B.Ns, P, B.sh.K, B.rchunks,
                                                           reinterpret_cast<const float2 *>(B.O), B.E, po, ps2, pf);
            k_moment_final<S><<<nb, kVecThreads, 0, st>>>(B.Ns, P, B.rchunks, B.sp, po, ps2, pf, B.eloc, B.o, B.skk,
                                                           B.f, B.err);
            return cudaGetLastError();
        }
    }
    k_moment_part<S, S><<<g, kVecThreads, 0, st>>>(B.Ns, P, B.sh.K, B.rchunks, B.O, B.E, po, ps2, pf);
    k_moment_final<S><<<nb, kVecThreads, 0, st>>>(B.Ns, P, B.rchunks, B.sp, po, ps2, pf, B.eloc, B.o, B.skk, B.f,
                                                   B.err);
    return cudaGetLastError();
}

template <class S> cudaError_t launch_minres_init(const SolveBufs<S> &B, cudaStream_t st) {
    const int nb = mr_blocks(B.sh.P);
    k_minres_init_vec<S><<<nb, kMrThreads, 0, st>>>(B);
    k_minres_init_scalar<S><<<1, 32, 0, st>>>(B);
    k_minres_first_v<S><<<nb, kMrThreads, 0, st>>>(B);
    return launch_lanczos_step(B, st);  // step 1; its QLP step runs in the first loop body
}

// u = O v then the row-chunk partials of O^H u. In the mixed form v must
// already be mirrored in B.v32.
template <class S> static cudaError_t launch_sv_passes(const SolveBufs<S> &B, const S *v, cudaStream_t st) {
    const int P = B.sh.P, nb = (P + kVecThreads - 1) / kVecThreads;
    const int rows_per_block = kVecThreads / 32;
    const int rb = (B.Ns + rows_per_block - 1) / rows_per_block;
    dim3 g(nb, B.rchunks);
    if (B.fact) {
        const cudaError_t e = launch_frows(B.F, B.v32, B.u32, st);
        return e != cudaSuccess ? e : launch_fcols(B.F, B.u32, B.ypart32, st);
    }
    if constexpr (std::is_same<S, double>::value) {
        if (B.fG) return launch_sv_fused(B.Ns, P, B.fG, B.fNB, B.svp, B.O, v, B.ysv, B.err, B.guard, st, B.o_split != 0);
    }
    k_sv_rows<S><<<rb, kVecThreads, 0, st>>>(B.Ns, P, B.O, v, B.u, B.guard);
    k_sv_cols<S><<<g, kVecThreads, 0, st>>>(B.Ns, P, B.rchunks, B.O, B.u, B.ypart, B.guard);
    return cudaGetLastError();
}

// Launch of a kernel that may start while its predecessor on `st` drains
// (it calls pdl_wait before reading anything).
template <class... KArgs, class... Args>
static cudaError_t launch_after(void (*kern)(KArgs...), int grid, int block, cudaStream_t st, Args &&...args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

template <class S> cudaError_t launch_lanczos_step(const SolveBufs<S> &B, cudaStream_t st) {
    const int nb = mr_blocks(B.sh.P);
    cudaError_t e = launch_sv_passes(B, B.v, st);
    if (e == cudaSuccess) e = launch_after(k_lanczos_a<S>, nb, kMrColThreads, st, B);
    if (e == cudaSuccess) e = launch_after(k_lanczos_b<S>, nb, kMrThreads, st, B);
    if (e == cudaSuccess) e = launch_after(k_lanczos_next<S>, nb, kMrThreads, st, B);
    return e;
}

template <class S> cudaError_t launch_qlp_step(const SolveBufs<S> &B, cudaStream_t st) {
    k_qlp_scalar<S><<<1, 32, 0, st>>>(B);
    const cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : launch_after(k_qlp_vectors<S>, mr_blocks(B.sh.P), kMrThreads, st, B);
}

template <class S> cudaError_t launch_sv_rows_only(const SolveBufs<S> &B, cudaStream_t st) {
    const int rows_per_block = kVecThreads / 32;
    const int rb = (B.Ns + rows_per_block - 1) / rows_per_block;
    if (B.fact)
        return launch_frows(B.F, B.v32, B.u32, st);
    else
        k_sv_rows<S><<<rb, kVecThreads, 0, st>>>(B.Ns, B.sh.P, B.O, B.v, B.u, B.guard);
    return cudaGetLastError();
}

template <class S> cudaError_t launch_sv_cols_only(const SolveBufs<S> &B, cudaStream_t st) {
    const int nb = (B.sh.P + kVecThreads - 1) / kVecThreads;
    dim3 g(nb, B.rchunks);
    if (B.fact)
        return launch_fcols(B.F, B.u32, B.ypart32, st);
    else
        k_sv_cols<S><<<g, kVecThreads, 0, st>>>(B.Ns, B.sh.P, B.rchunks, B.O, B.u, B.ypart, B.guard);
    return cudaGetLastError();
}

template <class S> cudaError_t launch_sv_only(const SolveBufs<S> &B, cudaStream_t st) {
    return launch_sv_passes(B, B.v, st);
}

template <class S> cudaError_t launch_moment_part_only(const SolveBufs<S> &B, cudaStream_t st) {
    const int P = B.sh.P, nb = (P + kVecThreads - 1) / kVecThreads;
    S *po = B.ypart;
    S *pf = B.ypart + size_t(B.rchunks) * P;
    double *ps2 = reinterpret_cast<double *>(B.ypart + size_t(2) * B.rchunks * P);
    dim3 g(nb, B.rchunks);
    if (B.fact) {
        float *fo = B.ypart32, *ff = fo + size_t(B.rchunks) * P, *fs = ff + size_t(B.rchunks) * P;
        return launch_fmoments(B.F, B.E, fo, ff, fs, st);
    }
    if constexpr (std::is_same<S, double>::value) {
        if (B.o_split) {
            k_moment_part_split<<<g, kVecThreads, 0, st>>>(B.Ns, P, B.sh.K, B.rchunks,
                                                           reinterpret_cast<const float2 *>(B.O), B.E, po, ps2, pf);
            return cudaGetLastError();
        }
    }
    k_moment_part<S, S><<<g, kVecThreads, 0, st>>>(B.Ns, P, B.sh.K, B.rchunks, B.O, B.E, po, ps2, pf);
    return cudaGetLastError();
}

template <class S> cudaError_t launch_apply_S(const SolveBufs<S> &B, const S *v, S *out, cudaStream_t st) {
    const int nb = mr_blocks(B.sh.P);
    k_ov_part<S><<<nb, kMrThreads, 0, st>>>(B.sh.P, B.o, v, B.ovpart);
    if (B.fact) k_to_f32<<<nb, kMrThreads, 0, st>>>(B.sh.P, reinterpret_cast<const double *>(v), B.v32);
    const cudaError_t e = launch_sv_passes(B, v, st);
    if (e != cudaSuccess) return e;
    k_apply_out<S><<<nb, kMrColThreads, 0, st>>>(B, v, out);
    return cudaGetLastError();
}

template <class S>
cudaError_t launch_update(const Shape &sh, const StepParams *sp, const S *x, cplx *a, cplx *b, cplx *w,
                          cudaStream_t st) {
    k_update<S><<<(sh.P + 255) / 256, 256, 0, st>>>(sh, sp, x, a, b, w);
    return cudaGetLastError();
}

#define NQES_INST(S)                                                                                     \
    template cudaError_t launch_moments<S>(const SolveBufs<S> &, cudaStream_t);                          \
    template cudaError_t launch_minres_init<S>(const SolveBufs<S> &, cudaStream_t);                      \
    template cudaError_t launch_lanczos_step<S>(const SolveBufs<S> &, cudaStream_t);                     \
    template cudaError_t launch_qlp_step<S>(const SolveBufs<S> &, cudaStream_t);                         \
    template cudaError_t launch_apply_S<S>(const SolveBufs<S> &, const S *, S *, cudaStream_t);          \
    template cudaError_t launch_sv_rows_only<S>(const SolveBufs<S> &, cudaStream_t);                     \
    template cudaError_t launch_sv_cols_only<S>(const SolveBufs<S> &, cudaStream_t);                     \
    template cudaError_t launch_sv_only<S>(const SolveBufs<S> &, cudaStream_t);                          \
    template cudaError_t launch_moment_part_only<S>(const SolveBufs<S> &, cudaStream_t);                 \
    template cudaError_t launch_update<S>(const Shape &, const StepParams *, const S *, cplx *, cplx *, \
                                          cplx *, cudaStream_t);                                         \
    template cudaError_t launch_lanczos_group<S>(const SolveBufs<S> *, const int *, int, int, cudaStream_t); \
    template cudaError_t launch_qlp_group<S>(const SolveBufs<S> *, const int *, int, int, cudaStream_t);
NQES_INST(double)
NQES_INST(cplx)

}  // namespace nqes
