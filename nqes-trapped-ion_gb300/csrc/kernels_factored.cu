// Factored S·v and moments of the mixed form (real arithmetic, FP32 data).
//
// The log-derivatives of a sample (code/rbm.cc:199-239, closed form) are, for
// state k and parameter p of the augmented (N+1) x (M+1) grid of that state,
//     O_{s,k,(i,j)} = sum_kk B_s(kk->k) sigma~_{s,kk,i} T~_{s,k,kk,j}
// with B_s(kk->k) = (Phi^-1)_{k,kk} Phi_{kk,k}, sigma~_{s,kk,i} = sigma_i of
// configuration kk (i < N) or 1 (i = N), T~_{s,k,kk,j} = tanh theta_j of
// configuration kk under RBM k (j < M) or 1 (j = M). Grid entry (i, j) is the
// weight w_ij, (i, M) the visible bias a_i, (N, j) the hidden bias b_j; (N, M)
// is unused. A sample therefore needs K^2 M tanh values and K^2 coefficients
// (the spins are stored anyway) instead of the P = K(N + M + NM) entries of O.
//
// With a "row" r = (s, kk) (a sample and one of its configurations) and, for
// state k, W_k / va_k / vb_k the w / a / b blocks of a parameter vector:
//   rows:    u_s = sum_k sum_kk B [ sum_j (vb_j + sum_i sigma_i W_ij) T_j + sum_i sigma_i va_i ]
//   columns: Y_k(i, j) = sum_r w_r sigma_{r,i} T_{r,j}, plus the a and b blocks
//            (w_r = u_s B, B, or E_loc,s B)
//   squares: sum_s O^2 = the column sum over the virtual rows (s, kk <= kk2)
//            with weight c B B', signs sigma sigma' (XOR of the spin words) and
//            T T' (c = 2 off the diagonal)
// Both passes are register-blocked products over the sample dimension: a
// thread keeps an RB x JB (rows) or IB x JB (columns) block of accumulators,
// the step's W_k (rows) or the rows' w T (columns) are staged in shared
// memory, and the +-1 signs come straight from the spin words. The rows pass
// costs K^2 N M fused multiply-adds per sample and reads K^2 M floats; the
// dense form read P = K(N + M + N M) floats per sample and pass.
//
// Column-type results are written as per-chunk partials in the P layout that
// the MINRES-QLP epilogue and the moment finalisation read; all sums run in a
// fixed order.
#include <algorithm>

#include "nqes_internal.h"

namespace nqes {

namespace {

constexpr int kThreads = 256;
constexpr int kJT = 8;       // j-threads per i group (columns)
constexpr int kGroups = kThreads / kJT;
// rows per double-buffered batch of the column kernel (at most 64 KB of tanh
// rows): the narrow tiles take 64 rows, halving the barriers per row
__host__ __device__ constexpr int cols_stage(int JB) { return JB >= 64 ? 8 : JB >= 16 ? (JB >= 32 ? 16 : 32) : 64; }
constexpr int kMaxN = 128;

__device__ __forceinline__ bool down_bit(const uint64_t *s, int i) { return (s[i >> 6] >> (i & 63)) & 1ULL; }

// +1 for spin up (bit clear), -1 for spin down (bit set); i < 128.
__device__ __forceinline__ float sgn(uint64_t b0, uint64_t b1, int i) {
    const uint64_t w = i < 64 ? b0 : b1;
    return __int_as_float(0x3f800000 | (int((w >> (i & 63)) & 1ULL) << 31));
}

// u_s = O_s . v. Block: kThreads / JT row groups x JT j-threads; a row group
// owns RB consecutive rows (s, kk), a j-thread the JB / 4 float4 column
// chunks q JT + tj (interleaved, so that the JT threads of a group read
// consecutive 16-byte pieces of a staged row: no bank conflicts). W_k is
// staged in chunks of F.ic rows of JT JB floats (zero beyond M).
template <int JT, int JB, int RB>
__device__ __forceinline__ void frows_body(const FactArgs &F, const float *__restrict__ v, float *__restrict__ u,
                                           const int bid) {
    extern __shared__ float4 smem4[];
    if (loop_guard_off(F.guard)) return;
    constexpr int WS = JT * JB, NG = kThreads / JT;
    const int N = F.N, M = F.M, K = F.K, NW = F.NW, L = N + M + N * M, MT = F.MT, KK = K * K, IC = F.ic;
    if (!dyn_smem_covers((size_t(IC) * WS + ((N + 3) & ~3) + WS + NG * RB) * sizeof(float)) || NW > 2) {
        if (threadIdx.x == 0) atomicOr(F.err, kErrLaunch);
        return;
    }
    float *sw = reinterpret_cast<float *>(smem4);  // IC x WS
    float *sva = sw + IC * WS;                     // N (rounded to 4)
    float *svb = sva + ((N + 3) & ~3);             // WS
    float *surow = svb + WS;                       // NG * RB
    const int tj = threadIdx.x & (JT - 1), rg = threadIdx.x / JT;
    const int spb = (NG * RB) / K;                 // samples per block
    const int rows_here = min(spb, F.Ns - bid * spb) * K;
    const int rl0 = rg * RB;                       // first local row of the group
    const size_t rbase = size_t(bid) * spb * K;
    const FastDiv dK = fast_div(unsigned(K));
    uint64_t b0[RB], b1[RB];
#pragma unroll
    for (int rb = 0; rb < RB; rb++) {
        const size_t r = rbase + min(rl0 + rb, max(rows_here - 1, 0));
        b0[rb] = F.spins[r * NW];
        b1[rb] = NW > 1 ? F.spins[r * NW + 1] : 0ULL;
    }
    float tot[RB];
#pragma unroll
    for (int rb = 0; rb < RB; rb++) tot[rb] = 0.f;
    for (int k = 0; k < K; k++) {
        const float *vk = v + size_t(k) * L;
        __syncthreads();
        for (int t = threadIdx.x; t < WS; t += kThreads) svb[t] = t < M ? vk[N + t] : 0.f;
        for (int t = threadIdx.x; t < N; t += kThreads) sva[t] = vk[t];
        __syncthreads();
        float z[RB][JB];
#pragma unroll
        for (int jb = 0; jb < JB; jb++) {
            const float b = svb[((jb >> 2) * JT + tj) * 4 + (jb & 3)];
#pragma unroll
            for (int rb = 0; rb < RB; rb++) z[rb][jb] = b;
        }
        for (int i0 = 0; i0 < N; i0 += IC) {
            const int ni = min(IC, N - i0);
            __syncthreads();
            for (int t = threadIdx.x; t < ni * WS; t += kThreads) {
                const int ii = t / WS, j = t - ii * WS;
                sw[t] = j < M ? vk[N + M + size_t(i0 + ii) * M + j] : 0.f;
            }
            __syncthreads();
            // the sign of spin i0 + ii of each row at bit 31 of cur: the 32-bit
            // word holding it, bit-reversed, shifted left by one per spin (two
            // integer operations a spin instead of a 64-bit shift and select)
            auto word_rev = [&](int rb, int w) -> uint32_t {
                const uint64_t x = w < 2 ? b0[rb] : b1[rb];
                return __brev(uint32_t((w & 1) ? (x >> 32) : x));
            };
            uint32_t cur[RB];
#pragma unroll
            for (int rb = 0; rb < RB; rb++) cur[rb] = word_rev(rb, i0 >> 5) << (i0 & 31);
            for (int ii = 0; ii < ni; ii++) {
                if (ii > 0 && ((i0 + ii) & 31) == 0) {
#pragma unroll
                    for (int rb = 0; rb < RB; rb++) cur[rb] = word_rev(rb, (i0 + ii) >> 5);
                }
                const float4 *wr = reinterpret_cast<const float4 *>(sw + ii * WS) + tj;
                float wv[JB];
#pragma unroll
                for (int q = 0; q < JB / 4; q++) {
                    const float4 x = wr[q * JT];
                    wv[4 * q] = x.x;
                    wv[4 * q + 1] = x.y;
                    wv[4 * q + 2] = x.z;
                    wv[4 * q + 3] = x.w;
                }
#pragma unroll
                for (int rb = 0; rb < RB; rb++) {
                    const float sg = __uint_as_float((cur[rb] & 0x80000000u) | 0x3f800000u);  // -1: spin down
                    cur[rb] <<= 1;
#pragma unroll
                    for (int jb = 0; jb < JB; jb++) z[rb][jb] = fmaf(sg, wv[jb], z[rb][jb]);
                }
            }
        }
        // the a block: sum_i sigma_i va_i over i = tj (mod JT)
        float a[RB];
#pragma unroll
        for (int rb = 0; rb < RB; rb++) a[rb] = 0.f;
        for (int i = tj; i < N; i += JT) {
            const float va = sva[i];
#pragma unroll
            for (int rb = 0; rb < RB; rb++) a[rb] = fmaf(sgn(b0[rb], b1[rb], i), va, a[rb]);
        }
        // dot with the row's tanh values, times B (rbase is a multiple of K: the
        // row's sample and configuration from the local row alone)
#pragma unroll
        for (int rb = 0; rb < RB; rb++) {
            const int rl = rl0 + rb;
            if (rl < rows_here) {
                const unsigned sl = fdiv(unsigned(rl), dK);
                const size_t s = size_t(bid) * spb + sl;
                const int kk = rl - int(sl) * K, q = k * K + kk;
                const float *tr = F.T + (s * KK + q) * size_t(MT);
                float d = a[rb];
#pragma unroll
                for (int c = 0; c < JB / 4; c++) {
                    const int j = (c * JT + tj) * 4;
                    if (j < MT) {
                        const float4 x = __ldg(reinterpret_cast<const float4 *>(tr + j));
                        d = fmaf(z[rb][4 * c], x.x, d);
                        d = fmaf(z[rb][4 * c + 1], x.y, d);
                        d = fmaf(z[rb][4 * c + 2], x.z, d);
                        d = fmaf(z[rb][4 * c + 3], x.w, d);
                    }
                }
                tot[rb] = fmaf(__ldg(F.B + s * KK + q), d, tot[rb]);
            }
        }
    }
    // sum over the j-threads of the group, then over the configurations
#pragma unroll
    for (int rb = 0; rb < RB; rb++) {
#pragma unroll
        for (int o = 1; o < JT; o <<= 1) tot[rb] += __shfl_xor_sync(0xffffffffu, tot[rb], o);
        if (tj == 0) surow[rl0 + rb] = tot[rb];
    }
    __syncthreads();
    for (int sl = threadIdx.x; sl * K < rows_here; sl += kThreads) {
        float acc = 0.f;
        for (int kk = 0; kk < K; kk++) acc += surow[sl * K + kk];
        u[size_t(bid) * spb + sl] = acc;
    }
}
template <int JT, int JB, int RB>
__global__ void __launch_bounds__(kThreads, RB <= 2 ? 3 : 2) k_frows(FactArgs F, const float *__restrict__ v,
                                                                     float *__restrict__ u) {
    frows_body<JT, JB, RB>(F, v, u, blockIdx.x);
}
// The rows pass of a group of solves (one launch; group_member maps blocks to solves).
template <int JT, int JB, int RB>
__global__ void __launch_bounds__(kThreads, RB <= 2 ? 3 : 2) k_frows_g(const FactMember *__restrict__ tab,
                                                                       const int *__restrict__ first, int n) {
    const int m = group_member(first, n, blockIdx.x);
    const FactMember &fm = tab[m];
    frows_body<JT, JB, RB>(fm.F, fm.v32, fm.u32, int(blockIdx.x) - __ldg(first + m));
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Staging buffers, then weights and sign words; with row sets the staging
// buffers must also hold every thread's IB JB + IB + JB sums.
template <int IB, int JB> __host__ __device__ constexpr size_t cols_smem(bool sets) {
    constexpr size_t st = cols_stage(JB);
    constexpr size_t stage = size_t(2) * 2 * st * kJT * JB, red = size_t(kThreads) * (IB * JB + IB + JB);
    return ((sets && red > stage ? red : stage) + 2 * st) * sizeof(float) + size_t(2) * st * 2 * 8;
}

// Column-type partial sums over chunk blockIdx.x of the rows of state
// k = blockIdx.y, grid rows i in block blockIdx.z (kGroups * IB of them).
//   mode 0: w_r = u_s B          (the O^T u pass of S·v)
//   mode 1: w_r = B              (sum of O)
//   mode 2: w_r = E_loc,s B      (sum of E_loc O)
//   mode 3: squares: virtual rows (s, kk <= kk2), w = c B B', T T', XOR'ed signs
// out gets the chunk's partial in the P layout at out + chunk * P.
// Batches of cols_stage(JB) rows are double-buffered: the tanh rows of the next batch
// stream into shared memory (cp.async) and its weights and sign words are
// formed while the current batch is summed.
// Row sets: gn i groups cover the block's gn IB grid rows; the kGroups / gn
// sets of groups take every nset-th staged row, so a staged tanh row is read by
// gn groups instead of kGroups, and the sets' sums meet in shared memory at the
// end (in set order).
template <int IB, int JB>
__device__ __forceinline__ void fcols_body(const FactArgs &F, int mode, int gn, const float *__restrict__ w,
                                           const cplx *__restrict__ E, float *__restrict__ out, const int bx,
                                           const int by, const int bz) {
    if (loop_guard_off(F.guard)) return;
    constexpr int WS = kJT * JB, kStage = cols_stage(JB);
    extern __shared__ float4 smem4[];
    float *st = reinterpret_cast<float *>(smem4);          // [2][kStage][WS] tanh rows (second factor: [2][kStage][WS])
    float *sw1 = st + 2 * 2 * kStage * WS;                 // [2][kStage]
    uint64_t *sb = reinterpret_cast<uint64_t *>(sw1 + 2 * kStage);  // [2][kStage][2]
    const int N = F.N, M = F.M, K = F.K, NW = F.NW, L = N + M + N * M, MT = F.MT, KK = K * K;
    const int P = K * L;
    const int c = bx, k = by;
    const int tj = threadIdx.x & (kJT - 1), ig = threadIdx.x / kJT;
    const int nset = kGroups / gn, set = ig / gn, igl = ig - set * gn;
    if (!dyn_smem_covers(cols_smem<IB, JB>(nset > 1)) || NW > 2 || MT > WS) {
        if (threadIdx.x == 0) atomicOr(F.err, kErrLaunch);
        return;
    }
    const int ibase = bz * (gn * IB) + igl * IB;
    const int vpr = mode == 3 ? K * (K + 1) / 2 : K;  // (virtual) rows per sample
    const size_t nrows = size_t(F.Ns) * vpr;
    const size_t r0 = nrows * c / F.rchunks, r1 = nrows * (c + 1) / F.rchunks;
    const int nbat = int((r1 - r0 + kStage - 1) / kStage);
    const int nf = mode == 3 ? 2 : 1;
    // row -> (sample, configuration) and piece -> (row, 16 bytes) by high
    // multiplies while the row indices fit (uniform over the launch)
    const FastDiv dvpr = fast_div(unsigned(vpr)), dper = fast_div(unsigned(MT / 4));
    const bool fast = nrows < (size_t(1) << 32) / size_t(vpr);
    auto sample_of = [&](size_t r) -> size_t { return fast ? size_t(fdiv(unsigned(r), dvpr)) : r / vpr; };
    // zero the column padding of all buffers once (copies write [0, MT) only)
    for (int t = threadIdx.x; t < 2 * 2 * kStage * WS; t += kThreads) st[t] = 0.f;
    __syncthreads();

    // issue batch b into buffer b & 1: tanh rows by cp.async, weights and signs directly
    auto issue = [&](int bi) {
        const int buf = bi & 1;
        const size_t rb0 = r0 + size_t(bi) * kStage;
        const int nb = int(min(size_t(kStage), r1 - rb0));
        const int per = MT / 4;  // 16-byte pieces per row
        for (int t = threadIdx.x; t < nf * nb * per; t += kThreads) {
            const int f = t >= nb * per ? 1 : 0, rem = t - f * nb * per;
            const int rr = int(fdiv(unsigned(rem), dper)), pc = rem - rr * per;
            const size_t r = rb0 + rr, s = sample_of(r);
            int kk = int(r - s * vpr), kk2 = kk;
            if (mode == 3) {
                int a = 0;
                while (kk >= K - a) {
                    kk -= K - a;
                    a++;
                }
                kk2 = a + kk;
                kk = a;
            }
            const size_t row = s * KK + size_t(k) * K + (f == 0 ? kk : kk2);
            cp_async16(st + ((f * 2 + buf) * kStage + rr) * WS + 4 * pc, F.T + row * MT + 4 * pc);
        }
        cp_async_commit();
        if (threadIdx.x < nb) {
            const int rr = threadIdx.x;
            const size_t r = rb0 + rr, s = sample_of(r);
            int kk = int(r - s * vpr), kk2 = -1;
            if (mode == 3) {
                int a = 0;
                while (kk >= K - a) {
                    kk -= K - a;
                    a++;
                }
                kk2 = a + kk;
                kk = a;
            }
            const size_t qo = s * KK + size_t(k) * K;
            float wr = __ldg(F.B + qo + kk);
            if (mode == 0) wr *= __ldg(w + s);
            if (mode == 2) {
                double el = 0.0;
                for (int q = 0; q < K; q++) el += E[s * KK + q * K + q].re;
                wr *= float(el);
            }
            uint64_t x0 = F.spins[(s * K + kk) * NW], x1 = NW > 1 ? F.spins[(s * K + kk) * NW + 1] : 0ULL;
            if (mode == 3) {
                wr *= (kk == kk2 ? 1.f : 2.f) * __ldg(F.B + qo + kk2);
                x0 ^= F.spins[(s * K + kk2) * NW];
                if (NW > 1) x1 ^= F.spins[(s * K + kk2) * NW + 1];
            }
            sw1[buf * kStage + rr] = wr;
            sb[(buf * kStage + rr) * 2] = x0;
            sb[(buf * kStage + rr) * 2 + 1] = x1;
        }
    };

    float acc[IB][JB], acca[IB], accb[JB];
#pragma unroll
    for (int ii = 0; ii < IB; ii++) {
        acca[ii] = 0.f;
#pragma unroll
        for (int jb = 0; jb < JB; jb++) acc[ii][jb] = 0.f;
    }
#pragma unroll
    for (int jb = 0; jb < JB; jb++) accb[jb] = 0.f;
    const bool bgroup = bz == 0 && igl == 0;
    // the thread's IB grid rows share one 32-bit half of the sign words (IB | 32):
    // a sign is that word shifted so the row's bit is the top bit, XORed into the weight
    const uint32_t *sb32 = reinterpret_cast<const uint32_t *>(sb);
    const int ib_c = min(ibase, kMaxN - IB), wsel = ib_c >> 5, sh0 = ib_c & 31;
    if (nbat > 0) issue(0);
    for (int bi = 0; bi < nbat; bi++) {
        const int buf = bi & 1;
        const int nb = int(min(size_t(kStage), r1 - (r0 + size_t(bi) * kStage)));
        if (bi + 1 < nbat) {
            issue(bi + 1);
        } else {
            cp_async_commit();  // an empty group keeps the wait count uniform
        }
        cp_async_wait1();
        __syncthreads();
        const float *tb = st + (size_t(buf) * kStage) * WS, *tb2 = st + (size_t(2 + buf) * kStage) * WS;
        for (int rr = set; rr < nb; rr += nset) {
            float tv[JB];
            const float4 *tp = reinterpret_cast<const float4 *>(tb + rr * WS) + tj;
#pragma unroll
            for (int q = 0; q < JB / 4; q++) {
                const float4 x = tp[q * kJT];
                tv[4 * q] = x.x;
                tv[4 * q + 1] = x.y;
                tv[4 * q + 2] = x.z;
                tv[4 * q + 3] = x.w;
            }
            if (mode == 3) {
                const float4 *tp2 = reinterpret_cast<const float4 *>(tb2 + rr * WS) + tj;
#pragma unroll
                for (int q = 0; q < JB / 4; q++) {
                    const float4 x = tp2[q * kJT];
                    tv[4 * q] *= x.x;
                    tv[4 * q + 1] *= x.y;
                    tv[4 * q + 2] *= x.z;
                    tv[4 * q + 3] *= x.w;
                }
            }
            const float wr = sw1[buf * kStage + rr];
            const uint32_t wd = sb32[(buf * kStage + rr) * 4 + wsel];
#pragma unroll
            for (int ii = 0; ii < IB; ii++) {
                const uint32_t sbit = (wd << (31 - (sh0 + ii))) & 0x80000000u;  // bit set: spin down
                const float sw = __uint_as_float(__float_as_uint(wr) ^ sbit);
#pragma unroll
                for (int jb = 0; jb < JB; jb++) acc[ii][jb] = fmaf(sw, tv[jb], acc[ii][jb]);
            }
            if (bgroup) {
#pragma unroll
                for (int jb = 0; jb < JB; jb++) accb[jb] = fmaf(wr, tv[jb], accb[jb]);
            }
        }
        // the a block: the set's rows, one in kJT per j-thread
        for (int rr = set + nset * tj; rr < nb; rr += nset * kJT) {
            const float wr = sw1[buf * kStage + rr];
            const uint32_t wd = sb32[(buf * kStage + rr) * 4 + wsel];
#pragma unroll
            for (int ii = 0; ii < IB; ii++)
                acca[ii] += __uint_as_float(__float_as_uint(wr) ^ ((wd << (31 - (sh0 + ii))) & 0x80000000u));
        }
        __syncthreads();  // buffer buf is refilled by the next issue
    }
#pragma unroll
    for (int ii = 0; ii < IB; ii++)
#pragma unroll
        for (int o = 1; o < kJT; o <<= 1) acca[ii] += __shfl_xor_sync(0xffffffffu, acca[ii], o);
    if constexpr (JB < 32) {  // wider tiles run as one set
      if (nset > 1) {
        // sets 1.. hand their sums to set 0 through the (now idle) staging buffers:
        // value v of thread t at red[v * kThreads + t]
        constexpr int R = IB * JB + IB + JB;
        float *red = st;
#pragma unroll
        for (int ii = 0; ii < IB; ii++) {
#pragma unroll
            for (int jb = 0; jb < JB; jb++) red[(ii * JB + jb) * kThreads + threadIdx.x] = acc[ii][jb];
            red[(IB * JB + ii) * kThreads + threadIdx.x] = acca[ii];
        }
#pragma unroll
        for (int jb = 0; jb < JB; jb++) red[(IB * JB + IB + jb) * kThreads + threadIdx.x] = accb[jb];
        __syncthreads();
        if (set != 0) return;
        for (int s2 = 1; s2 < nset; s2++) {
            const int t2 = threadIdx.x + s2 * gn * kJT;
#pragma unroll
            for (int ii = 0; ii < IB; ii++) {
#pragma unroll
                for (int jb = 0; jb < JB; jb++) acc[ii][jb] += red[(ii * JB + jb) * kThreads + t2];
                acca[ii] += red[(IB * JB + ii) * kThreads + t2];
            }
#pragma unroll
            for (int jb = 0; jb < JB; jb++) accb[jb] += red[(IB * JB + IB + jb) * kThreads + t2];
        }
        static_assert(R > 0, "reduction layout");
      }
    }
    float *o = out + size_t(c) * P + size_t(k) * L;
#pragma unroll
    for (int ii = 0; ii < IB; ii++) {
        const int i = ibase + ii;
        if (i < N) {
#pragma unroll
            for (int jb = 0; jb < JB; jb++) {
                const int j = ((jb >> 2) * kJT + tj) * 4 + (jb & 3);
                if (j < M) o[N + M + size_t(i) * M + j] = acc[ii][jb];
            }
            if (tj == 0) o[i] = acca[ii];
        }
    }
    if (bgroup) {
#pragma unroll
        for (int jb = 0; jb < JB; jb++) {
            const int j = ((jb >> 2) * kJT + tj) * 4 + (jb & 3);
            if (j < M) o[N + j] = accb[jb];
        }
    }
}
template <int IB, int JB>
__global__ void __launch_bounds__(kThreads, 2) k_fcols(FactArgs F, int mode, int gn, const float *__restrict__ w,
                                                     const cplx *__restrict__ E, float *__restrict__ out) {
    fcols_body<IB, JB>(F, mode, gn, w, E, out, blockIdx.x, blockIdx.y, blockIdx.z);
}
// The O^T u pass (mode 0) of a group of solves: solve m's blocks in the order
// of its own (rchunks, K, i blocks) grid.
template <int IB, int JB>
__global__ void __launch_bounds__(kThreads, 2) k_fcols_g(const FactMember *__restrict__ tab,
                                                       const int *__restrict__ first, int n) {
    const int m = group_member(first, n, blockIdx.x);
    const FactMember &fm = tab[m];
    const int lin = int(blockIdx.x) - __ldg(first + m), X = fm.F.rchunks, Y = fm.F.K;
    fcols_body<IB, JB>(fm.F, 0, fm.gn, fm.u32, nullptr, fm.ypart32, lin % X, (lin / X) % Y, lin / (X * Y));
}

// o, skk = reglam (<O^2> - o^2), f = <E_loc O> - eloc o from the chunk partials.
__global__ void k_fmoment_final(int Ns, int P, int rchunks, const StepParams *sp, const float *po, const float *pf,
                                const float *ps2, const cplx *eloc, double *o, double *skk, double *f, int *err) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    double so = 0.0, sf = 0.0, s2 = 0.0;
    for (int r = 0; r < rchunks; r++) {
        so += po[size_t(r) * P + p];
        sf += pf[size_t(r) * P + p];
        s2 += ps2[size_t(r) * P + p];
    }
    const double inv = 1.0 / double(Ns), om = so * inv;
    const double dg = (s2 * inv - om * om) * sp->reglam;
    const double fv = sf * inv - eloc[0].re * om;
    o[p] = om;
    skk[p] = dg;
    f[p] = fv;
    if (!isfinite(om) || !isfinite(dg) || !isfinite(fv)) atomicOr(err, kErrNonFinite);
}

// Rows [first, first + count) of O from the factors (for inspection).
__global__ void k_fO(FactArgs F, int first, int count, float *O) {
    const int N = F.N, M = F.M, K = F.K, NW = F.NW, L = N + M + N * M, P = K * L, KK = K * K;
    const size_t total = size_t(count) * P;
    for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < total; e += size_t(gridDim.x) * blockDim.x) {
        const size_t s = size_t(first) + e / P;
        const int p = int(e % P), k = p / L, q = p - k * L;
        int i, j;
        if (q < N) {
            i = q;
            j = M;
        } else if (q < N + M) {
            i = N;
            j = q - N;
        } else {
            i = (q - N - M) / M;
            j = (q - N - M) - i * M;
        }
        float v = 0.f;
        for (int kk = 0; kk < K; kk++) {
            const float b = F.B[s * KK + k * K + kk];
            const float tt = j < M ? F.T[(s * KK + k * K + kk) * F.MT + j] : 1.f;
            const bool dn = i < N && down_bit(F.spins + (s * K + kk) * NW, i);
            v += dn ? -b * tt : b * tt;
        }
        O[e] = v;
    }
}

// Launch shapes. Rows: JT j-threads of JB columns (JT JB >= M), RB rows per
// row group (RB JB <= 64, <= 32 below 16 columns). Columns: kJT j-threads of
// JB columns, IB grid rows per i group (IB JB <= 64, <= 32 from 32 columns).
int pick_jb(int M) {
    const int jb = (M + kJT - 1) / kJT;
    return jb <= 4 ? 4 : jb <= 8 ? 8 : jb <= 16 ? 16 : jb <= 32 ? 32 : 64;
}
// Grid rows per thread of the column kernel: 4 where JB <= 16 and N needs them
// (each staged tanh value then feeds 4 FMAs), 1 beyond.
int pick_ib(int N, int JB) {
    if (JB >= 32) return 1;
    return N <= 1 ? 1 : N <= 2 ? 2 : 4;
}
// i groups per row set: the smallest power of two covering N with IB rows each
// (capped at kGroups); with JB >= 32 every group covers rows (one set), since
// the sets' sums would not fit the shared memory of two blocks per SM.
int pick_gn(int N, int IB, int JB) {
    if (JB >= 32) return kGroups;
    const int need = (N + IB - 1) / IB;
    int gn = 1;
    while (gn < need && gn < kGroups) gn <<= 1;
    return gn;
}
template <int JT, int JB, int RB0 = 0>
cudaError_t rows_launch(FactArgs F, const float *v, float *u, cudaStream_t st, bool prepare) {
    constexpr int RB = RB0 ? RB0 : JB >= 16 ? 64 / JB : 32 / JB, WS = JT * JB, NG = kThreads / JT;
    F.ic = std::max(1, std::min(F.N, (48 * 1024 / 4) / WS));
    const size_t smem = (size_t(F.ic) * WS + ((F.N + 3) & ~3) + WS + NG * RB) * sizeof(float);
    if (prepare)
        return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_frows<JT, JB, RB>));
    const int spb = (NG * RB) / F.K;
    const int blocks = (F.Ns + spb - 1) / spb;
    k_frows<JT, JB, RB><<<blocks, kThreads, smem, st>>>(F, v, u);
    return cudaGetLastError();
}
cudaError_t rows_dispatch(const FactArgs &F, const float *v, float *u, cudaStream_t st, bool prepare) {
    const int M = F.M;
    if (M <= 16) return rows_launch<4, 4>(F, v, u, st, prepare);
    if (M <= 32) return rows_launch<4, 8>(F, v, u, st, prepare);
    if (M <= 64) return rows_launch<4, 16, 2>(F, v, u, st, prepare);  // 2 rows a group: 3 blocks per SM
    if (M <= 128) return rows_launch<8, 16>(F, v, u, st, prepare);
    if (M <= 256) return rows_launch<8, 32>(F, v, u, st, prepare);
    return rows_launch<8, 64>(F, v, u, st, prepare);
}

template <int IB, int JB>
cudaError_t cols_launch(const FactArgs &F, int mode, const float *w, const cplx *E, float *out, cudaStream_t st,
                        bool prepare) {
    const int gn = pick_gn(F.N, IB, JB);
    const size_t smem = cols_smem<IB, JB>(gn < kGroups);
    if (prepare) return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_fcols<IB, JB>));
    dim3 g(F.rchunks, F.K, (F.N + gn * IB - 1) / (gn * IB));
    k_fcols<IB, JB><<<g, kThreads, smem, st>>>(F, mode, gn, w, E, out);
    return cudaGetLastError();
}
template <int JB>
cudaError_t cols_ib(const FactArgs &F, int mode, const float *w, const cplx *E, float *out, cudaStream_t st,
                    bool prepare) {
    switch (pick_ib(F.N, JB)) {
    case 1: return cols_launch<1, JB>(F, mode, w, E, out, st, prepare);
    case 2:
        if constexpr (JB < 32) return cols_launch<2, JB>(F, mode, w, E, out, st, prepare);
        return cudaErrorInvalidConfiguration;
    default:
        if constexpr (4 * JB <= 64) return cols_launch<4, JB>(F, mode, w, E, out, st, prepare);
        return cudaErrorInvalidConfiguration;
    }
}
cudaError_t cols_dispatch(const FactArgs &F, int mode, const float *w, const cplx *E, float *out, cudaStream_t st,
                          bool prepare = false) {
    switch (pick_jb(F.M)) {
    case 4: return cols_ib<4>(F, mode, w, E, out, st, prepare);
    case 8: return cols_ib<8>(F, mode, w, E, out, st, prepare);
    case 16: return cols_ib<16>(F, mode, w, E, out, st, prepare);
    case 32: return cols_ib<32>(F, mode, w, E, out, st, prepare);
    default: return cols_ib<64>(F, mode, w, E, out, st, prepare);
    }
}

// Grouped launches: variant ids. Rows: the case of rows_dispatch (by M);
// columns: 10 JB + IB.
template <int JT, int JB, int RB0 = 0>
cudaError_t rows_group(const FactMember *tab, const int *first, int n, int blocks, size_t smem, cudaStream_t st,
                       bool prepare) {
    constexpr int RB = RB0 ? RB0 : JB >= 16 ? 64 / JB : 32 / JB;
    if (prepare) return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_frows_g<JT, JB, RB>));
    k_frows_g<JT, JB, RB><<<blocks, kThreads, smem, st>>>(tab, first, n);
    return cudaGetLastError();
}
cudaError_t rows_group_dispatch(int variant, const FactMember *tab, const int *first, int n, int blocks, size_t smem,
                                cudaStream_t st, bool prepare) {
    switch (variant) {
    case 0: return rows_group<4, 4>(tab, first, n, blocks, smem, st, prepare);
    case 1: return rows_group<4, 8>(tab, first, n, blocks, smem, st, prepare);
    case 2: return rows_group<4, 16, 2>(tab, first, n, blocks, smem, st, prepare);
    case 3: return rows_group<8, 16>(tab, first, n, blocks, smem, st, prepare);
    case 4: return rows_group<8, 32>(tab, first, n, blocks, smem, st, prepare);
    case 5: return rows_group<8, 64>(tab, first, n, blocks, smem, st, prepare);
    case 6: return rows_group<4, 16, 4>(tab, first, n, blocks, smem, st, prepare);  // case 2, 4 rows a group
    default: return cudaErrorInvalidValue;
    }
}
template <int IB, int JB>
cudaError_t cols_group(const FactMember *tab, const int *first, int n, int blocks, size_t smem, cudaStream_t st,
                       bool prepare) {
    if (prepare) return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_fcols_g<IB, JB>));
    k_fcols_g<IB, JB><<<blocks, kThreads, smem, st>>>(tab, first, n);
    return cudaGetLastError();
}
cudaError_t cols_group_dispatch(int variant, const FactMember *tab, const int *first, int n, int blocks, size_t smem,
                                cudaStream_t st, bool prepare) {
    switch (variant) {
    case 41: return cols_group<1, 4>(tab, first, n, blocks, smem, st, prepare);
    case 42: return cols_group<2, 4>(tab, first, n, blocks, smem, st, prepare);
    case 44: return cols_group<4, 4>(tab, first, n, blocks, smem, st, prepare);
    case 81: return cols_group<1, 8>(tab, first, n, blocks, smem, st, prepare);
    case 82: return cols_group<2, 8>(tab, first, n, blocks, smem, st, prepare);
    case 84: return cols_group<4, 8>(tab, first, n, blocks, smem, st, prepare);
    case 161: return cols_group<1, 16>(tab, first, n, blocks, smem, st, prepare);
    case 162: return cols_group<2, 16>(tab, first, n, blocks, smem, st, prepare);
    case 164: return cols_group<4, 16>(tab, first, n, blocks, smem, st, prepare);
    case 321: return cols_group<1, 32>(tab, first, n, blocks, smem, st, prepare);
    case 641: return cols_group<1, 64>(tab, first, n, blocks, smem, st, prepare);
    default: return cudaErrorInvalidValue;
    }
}
// Shared memory of the column kernel for (IB, JB) with or without row sets.
size_t cols_smem_of(int IB, int JB, bool sets) {
    switch (JB) {
    case 4: return IB == 1 ? cols_smem<1, 4>(sets) : IB == 2 ? cols_smem<2, 4>(sets) : cols_smem<4, 4>(sets);
    case 8: return IB == 1 ? cols_smem<1, 8>(sets) : IB == 2 ? cols_smem<2, 8>(sets) : cols_smem<4, 8>(sets);
    case 16: return IB == 1 ? cols_smem<1, 16>(sets) : IB == 2 ? cols_smem<2, 16>(sets) : cols_smem<4, 16>(sets);
    case 32: return cols_smem<1, 32>(sets);
    default: return cols_smem<1, 64>(sets);
    }
}

}  // namespace

void fact_rows_geometry(int variant, const FactArgs &F, int *blocks, size_t *smem, int *ic) {
    int JT, JB, RB;
    switch (variant) {
    case 0: JT = 4; JB = 4; RB = 32 / 4; break;
    case 1: JT = 4; JB = 8; RB = 32 / 8; break;
    case 2: JT = 4; JB = 16; RB = 2; break;
    case 3: JT = 8; JB = 16; RB = 64 / 16; break;
    case 4: JT = 8; JB = 32; RB = 64 / 32; break;
    case 6: JT = 4; JB = 16; RB = 4; break;
    default: JT = 8; JB = 64; RB = 64 / 64; break;
    }
    // as rows_launch
    const int WS = JT * JB, NG = kThreads / JT;
    *ic = std::max(1, std::min(F.N, (48 * 1024 / 4) / WS));
    *smem = (size_t(*ic) * WS + ((F.N + 3) & ~3) + WS + NG * RB) * sizeof(float);
    const int spb = (NG * RB) / F.K;
    *blocks = (F.Ns + spb - 1) / spb;
}

FactGroupPlan fact_group_plan(const FactArgs &F) {
    FactGroupPlan g{};
    const int M = F.M;
    g.rows_variant = M <= 16 ? 0 : M <= 32 ? 1 : M <= 64 ? 2 : M <= 128 ? 3 : M <= 256 ? 4 : 5;
    fact_rows_geometry(g.rows_variant, F, &g.rows_blocks, &g.rows_smem, &g.ic);
    // as cols_dispatch / cols_launch
    const int cjb = pick_jb(F.M), cib = pick_ib(F.N, cjb);
    g.cols_variant = 10 * cjb + cib;
    g.gn = pick_gn(F.N, cib, cjb);
    g.cols_smem = cols_smem_of(cib, cjb, g.gn < kGroups);
    g.zg = (F.N + g.gn * cib - 1) / (g.gn * cib);
    g.cols_blocks = F.rchunks * F.K * g.zg;
    return g;
}

cudaError_t prepare_fact_group(const FactGroupPlan &g) {
    cudaError_t e = rows_group_dispatch(g.rows_variant, nullptr, nullptr, 0, 0, 0, nullptr, true);
    return e != cudaSuccess ? e : cols_group_dispatch(g.cols_variant, nullptr, nullptr, 0, 0, 0, nullptr, true);
}

cudaError_t launch_frows_group(int variant, const FactMember *tab, const int *first, int n, int blocks, size_t smem,
                               cudaStream_t st) {
    return rows_group_dispatch(variant, tab, first, n, blocks, smem, st, false);
}

cudaError_t launch_fcols_group(int variant, const FactMember *tab, const int *first, int n, int blocks, size_t smem,
                               cudaStream_t st) {
    return cols_group_dispatch(variant, tab, first, n, blocks, smem, st, false);
}

// Sets the rows and column kernels' shared-memory limits; call outside stream capture.
cudaError_t prepare_frows(const FactArgs &F) {
    cudaError_t e = rows_dispatch(F, nullptr, nullptr, nullptr, true);
    if (e == cudaSuccess) e = cols_dispatch(F, 0, nullptr, nullptr, nullptr, nullptr, true);
    if (e == cudaSuccess) e = prepare_frows_tc(F);
    if (e == cudaSuccess) e = prepare_fcols_tc();
    return e;
}

cudaError_t launch_frows(const FactArgs &F, const float *v, float *u, cudaStream_t st) {
    if (F.tc) return launch_frows_tc(F, v, u, F.err, st);
    return rows_dispatch(F, v, u, st, false);
}

cudaError_t launch_fcols(const FactArgs &F, const float *w, float *ypart, cudaStream_t st) {
    if (F.tcc) return launch_fcols_tc(F, 0, w, nullptr, ypart, F.err, st);
    return cols_dispatch(F, 0, w, nullptr, ypart, st);
}

cudaError_t launch_fmoments(const FactArgs &F, const cplx *E, float *po, float *pf, float *ps2, cudaStream_t st) {
    auto one = [&](int mode, const cplx *e, float *out) {
        return F.tcc ? launch_fcols_tc(F, mode, nullptr, e, out, F.err, st) : cols_dispatch(F, mode, nullptr, e, out, st);
    };
    cudaError_t e = one(1, nullptr, po);
    if (e == cudaSuccess) e = one(2, E, pf);
    if (e == cudaSuccess) e = one(3, nullptr, ps2);
    return e;
}

cudaError_t launch_fmoment_final(const FactArgs &F, const StepParams *sp, const float *po, const float *pf,
                                 const float *ps2, const cplx *eloc, double *o, double *skk, double *f, int *err,
                                 cudaStream_t st) {
    const int P = F.K * (F.N + F.M + F.N * F.M);
    k_fmoment_final<<<(P + 255) / 256, 256, 0, st>>>(F.Ns, P, F.rchunks, sp, po, pf, ps2, eloc, o, skk, f, err);
    return cudaGetLastError();
}

cudaError_t launch_fO(const FactArgs &F, int first, int count, float *O, cudaStream_t st) {
    k_fO<<<1024, 256, 0, st>>>(F, first, count, O);
    return cudaGetLastError();
}

}  // namespace nqes
