// Tensor-core (tcgen05) rows pass of the factored S·v: u = O v from the
// factors of O (kernels_factored.cu has the algebra and the FP32 CUDA-core
// form this one replaces where the shape allows).
//
// For state k and a tile of 128 rows r = (s, kk), the augmented product
//     D[r][j] = sum_i sigma~[r][i] Wt_k[j][i]
// with sigma~ = +-1 spin signs (i < N), 1 (i = N), 0 beyond, and Wt_k[j][i] =
// w_ij (i < N, j < M), vb_j (i = N, j < M), va_i (j = M, i < N), 0 beyond, gives
// D[r][j] = vb_j + sum_i sigma_i w_ij (j < M) and D[r][M] = sum_i sigma_i va_i, so
//     u_s = sum_{k, kk} B[s][k][kk] (sum_{j<M} D[r][j] T[r][j] + D[r][M]).
// A = sigma~ is exact in BF16. B = Wt_k is split into three BF16 terms
// (hi + mid + lo carry 24 significant bits), so three MMAs with FP32
// accumulation in tensor memory reproduce the FP32 product. The split image of
// Wt (all K states, K-major core-matrix layout) is built once per pass by
// k_rows_bimg and bulk-copied (cp.async.bulk on an mbarrier) into shared
// memory per state; thread r builds row r of A from the spin words and, after
// the MMAs complete, reads row r of D from tensor memory and contracts it
// with the row's tanh values. Waits are bounded (kErrTimeout).
#include <algorithm>

#include "nqes_internal.h"
#include "tc_util.cuh"

namespace nqes {

namespace {

constexpr int kTcThreads = 128;

struct RowsTcShape {
    int NP, MN;          // K extent (N + 1 rounded to 16), N extent (M + 1 rounded to 16)
    unsigned tcols;      // tensor-memory columns allocated (power of two >= 32, >= MN)
    size_t abytes, bbytes, smem;
};

RowsTcShape rows_tc_shape(const FactArgs &F) {
    RowsTcShape s{};
    s.NP = round16(F.N + 1);
    s.MN = round16(F.M + 1);
    s.tcols = 32;
    while (s.tcols < unsigned(s.MN)) s.tcols <<= 1;
    s.abytes = size_t(128) * s.NP * 2;
    s.bbytes = size_t(3) * s.MN * s.NP * 2;
    s.smem = s.abytes + s.bbytes + 64 + 128 * sizeof(float);
    // at most 512 / tcols CTAs per SM (tensor memory): ask for more than
    // per_sm / (n + 1) bytes each, so that at most n = 512 / tcols CTAs share an SM
    const size_t per_sm = 228 * 1024, cap = per_sm / (512 / s.tcols + 1) + 1024;
    s.smem = std::max(s.smem, std::min(cap, size_t(227 * 1024)));
    return s;
}

// Split image of Wt for every state: [k][split][K-major MN x NP] BF16.
__global__ void k_rows_bimg(FactArgs F, int NP, int MN, const float *__restrict__ v, uint16_t *__restrict__ img) {
    if (loop_guard_off(F.guard)) return;
    const int N = F.N, M = F.M, L = N + M + N * M;
    const size_t per = size_t(MN) * NP, total = size_t(F.K) * per;
    for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < total; e += size_t(gridDim.x) * blockDim.x) {
        const int k = int(e / per);
        const int rem = int(e - size_t(k) * per), j = rem / NP, i = rem - j * NP;
        const float *vk = v + size_t(k) * L;
        float x = 0.f;
        if (j < M && i < N)
            x = vk[N + M + size_t(i) * M + j];
        else if (j < M && i == N)
            x = vk[N + j];
        else if (j == M && i < N)
            x = vk[i];
        float r1, r2, r3;
        const uint16_t h1 = bf16_split(x, r1), h2 = bf16_split(r1, r2), h3 = bf16_split(r2, r3);
        const size_t o = kmajor_off(j, i, NP) / 2;
        uint16_t *b = img + size_t(k) * 3 * per;
        b[o] = h1;
        b[per + o] = h2;
        b[2 * per + o] = h3;
    }
}

__global__ void __launch_bounds__(kTcThreads) k_frows_tc(FactArgs F, int NP, int MN, unsigned tcols, size_t abytes,
                                                       size_t bbytes, const uint16_t *__restrict__ img,
                                                       float *__restrict__ u, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    if (loop_guard_off(F.guard)) return;  // before any barrier init or tensor-memory allocation
    if (!dyn_smem_covers(abytes + bbytes + 64 + kTcThreads * sizeof(float)) || unsigned(MN) > tcols || tcols > 512 ||
        F.NW > 2) {
        if (threadIdx.x == 0) atomicOr(err, kErrLaunch);
        return;
    }
    const int N = F.N, M = F.M, K = F.K, NW = F.NW, MT = F.MT, KK = K * K;
    unsigned char *sA = smem_raw;
    unsigned char *sB = smem_raw + abytes;
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sB + bbytes);  // [0] B copy, [1] MMAs done
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 2);
    int *sflag = reinterpret_cast<int *>(tslot + 1);
    float *srow = reinterpret_cast<float *>(mbar + 4);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int spt = kTcThreads / K;  // samples per tile
    const int ntiles = (F.Ns + spt - 1) / spt;
    if (tid == 0) {
        mbar_init(&mbar[0], 1);
        mbar_init(&mbar[1], 1);
        *sflag = 0;
    }
    if (warp == 0) tmem_alloc(tslot, tcols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    const uint32_t idesc = idesc_bf16_f32(128, MN);
    const unsigned sbo = unsigned(NP) * 16;
    unsigned ph0 = 0, ph1 = 0;
    bool copy_pend = false, mma_pend = false;  // thread 0: an operation it could not see complete
    unsigned copy_ph = 0, mma_ph = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const size_t s0 = size_t(tile) * spt;
        const int ns = min(spt, F.Ns - int(s0)), nr = ns * K;
        const bool live = tid < nr;
        const size_t r = s0 * K + tid;
        const size_t s = s0 + (live ? tid / K : 0);
        const int kk = live ? tid % K : 0;
        // row tid of A: spin signs, 1 at i = N, 0 beyond (and for idle rows)
        {
            uint64_t b0 = 0, b1 = 0;
            if (live) {
                b0 = F.spins[r * NW];
                b1 = NW > 1 ? F.spins[r * NW + 1] : 0ULL;
            }
            for (int c = 0; c < NP / 8; c++) {
                uint32_t wv[4];
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    uint32_t pr = 0;
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int i = c * 8 + h * 2 + e;
                        uint32_t val = 0;
                        if (live) {
                            if (i < N)
                                val = (((i < 64 ? b0 >> i : b1 >> (i - 64)) & 1ULL) ? 0xBF80u : 0x3F80u);
                            else if (i == N)
                                val = 0x3F80u;
                        }
                        pr |= val << (16 * e);
                    }
                    wv[h] = pr;
                }
                *reinterpret_cast<uint4 *>(sA + kmajor_off(tid, c * 8, NP)) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
            }
        }
        fence_async_smem();
        float tot = 0.f;
        for (int k = 0; k < K; k++) {
            tc_fence_before();
            __syncthreads();  // A written; the previous MMAs and tensor-memory reads are done
            bool issued = false;
            if (tid == 0) {
                mbar_expect_tx(&mbar[0], unsigned(bbytes));
                bulk_g2s(sB, img + size_t(k) * 3 * MN * NP, unsigned(bbytes), &mbar[0]);
                if (!mbar_wait(&mbar[0], ph0)) {
                    *sflag = 1;
                    copy_pend = true;
                    copy_ph = ph0;
                } else {
                    tc_fence_after();
#pragma unroll 1
                    for (int q = 0; q < 3; q++)
#pragma unroll 1
                        for (int ks = 0; ks < NP / 16; ks++) {
                            const uint64_t ad = smem_desc(sA + ks * 256, 128, sbo);
                            const uint64_t bd = smem_desc(sB + size_t(q) * MN * NP * 2 + ks * 256, 128, sbo);
                            mma_bf16(tbase, ad, bd, idesc, q > 0 || ks > 0);
                        }
                    mma_commit(&mbar[1]);
                    issued = true;
                }
            }
            ph0 ^= 1;
            __syncthreads();
            if (*sflag) break;
            const bool done = mbar_wait(&mbar[1], ph1);
            if (!done) {
                *sflag = 1;
                if (tid == 0 && issued) {
                    mma_pend = true;
                    mma_ph = ph1;
                }
            }
            ph1 ^= 1;
            __syncthreads();
            if (*sflag) break;
            tc_fence_after();
            // row tid of D against the row's tanh values
            const float *tr = F.T + (s * KK + size_t(k) * K + kk) * MT;
            float d = 0.f;
            for (int c0 = 0; c0 < MN; c0 += 16) {
                float dv[16];
                tmem_ld16(tbase + (uint32_t(32 * warp) << 16) + uint32_t(c0), dv);
                if (live) {
#pragma unroll
                    for (int q4 = 0; q4 < 4; q4++) {
                        const int j = c0 + 4 * q4;
                        if (j < MT) {
                            const float4 t4 = __ldg(reinterpret_cast<const float4 *>(tr + j));
                            d = fmaf(dv[4 * q4], t4.x, d);
                            d = fmaf(dv[4 * q4 + 1], t4.y, d);
                            d = fmaf(dv[4 * q4 + 2], t4.z, d);
                            d = fmaf(dv[4 * q4 + 3], t4.w, d);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < 16; q++)
                        if (c0 + q == M) d += dv[q];  // the a block (T is 0 in the padding)
                }
            }
            if (live) tot = fmaf(__ldg(F.B + s * KK + size_t(k) * K + kk), d, tot);
        }
        if (*sflag) break;
        srow[tid] = tot;
        __syncthreads();
        if (tid < ns) {
            float a = 0.f;
            for (int q = 0; q < K; q++) a += srow[tid * K + q];
            u[s0 + tid] = a;
        }
        __syncthreads();
    }
    if (tid == 0 && *sflag) {
        atomicOr(err, kErrTimeout);
        // operations still in flight get one more bounded wait before the
        // tensor memory and the shared memory are released
        if (copy_pend) mbar_wait(&mbar[0], copy_ph);
        if (mma_pend) mbar_wait(&mbar[1], mma_ph);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, tcols);
}


// ---- column pass on the tensor cores ----
//
// For state k = blockIdx.y and chunk blockIdx.x of the rows r (a sample and a
// configuration; mode 3: a sample and a pair of configurations), the augmented
//     D[i][j] = sum_r A[i][r] Bt[j][r]
// with A[i][r] = sigma_r[i] (i < N), 1 (i = N), 0 beyond, and Bt[j][r] =
// w_r T_r[j] (j < M), w_r (j = M), 0 beyond, holds the w block (i < N, j < M),
// the a block (i < N, j = M) and the b block (i = N, j < M) of the chunk's
// column sum. A is exact in BF16; Bt is split exactly into three BF16 terms
// by truncation (8 + 8 + 8 significant bits), so three MMAs per K step of 16
// rows with FP32 accumulation in tensor memory give the FP32 sums. Per batch
// of 64 rows the tanh rows stream into shared memory (cp.async) while the
// previous batch's MMAs run; the threads then write A (thread i: row i from
// the sign words) and Bt (thread j: row j from the staged tanh values) in the
// K-major core-matrix layout. The partial is read back from tensor memory at
// the end of the chunk.

constexpr int kColRows = 64;      // K extent of one batch
constexpr int kColThreadsTc = 256;

struct ColsTcShape {
    int MN;
    unsigned tcols;
    size_t tbytes, abytes, bbytes, smem;
};

// Shared memory: the tanh rows (two batches, or one batch of both factors for
// the squares), A, the three planes of Bt, and per batch weights and sign words.
ColsTcShape cols_tc_shape(const FactArgs &F) {
    ColsTcShape s{};
    s.MN = round16(F.M + 1);
    s.tcols = 32;
    while (s.tcols < unsigned(s.MN)) s.tcols <<= 1;
    s.tbytes = size_t(2) * kColRows * F.MT * 4;
    s.abytes = size_t(128) * kColRows * 2;
    s.bbytes = size_t(3) * s.MN * kColRows * 2;
    s.smem = s.tbytes + s.abytes + s.bbytes + 2 * kColRows * (4 + 16) + 64;
    // more than per_sm / (n + 1) each, so that at most n = 512 / tcols CTAs share an SM
    const size_t per_sm = 228 * 1024, cap = per_sm / (512 / s.tcols + 1) + 1024;
    s.smem = std::max(s.smem, std::min(cap, size_t(227 * 1024)));
    return s;
}

__device__ __forceinline__ void cp_async16_cg(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

__global__ void __launch_bounds__(kColThreadsTc) k_fcols_tc(FactArgs F, int mode, int MN, unsigned tcols,
                                                          size_t tbytes, size_t abytes, size_t bbytes,
                                                          const float *__restrict__ w, const cplx *__restrict__ E,
                                                          float *__restrict__ out, int *err) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    if (loop_guard_off(F.guard)) return;  // before any barrier init or tensor-memory allocation
    if (!dyn_smem_covers(tbytes + abytes + bbytes + 2 * kColRows * (4 + 16) + 16) || unsigned(MN) > tcols ||
        tcols > 512 || F.NW > 2) {
        if (threadIdx.x == 0) atomicOr(err, kErrLaunch);
        return;
    }
    const int N = F.N, M = F.M, K = F.K, NW = F.NW, L = N + M + N * M, MT = F.MT, KK = K * K, P = K * L;
    float *sT = reinterpret_cast<float *>(smem_raw);  // [2][rows][MT]: two batches, or (mode 3) two factors
    unsigned char *sA = smem_raw + tbytes;
    unsigned char *sB = sA + abytes;
    float *sw = reinterpret_cast<float *>(sB + bbytes);                 // [2][rows] weights
    uint64_t *sbits = reinterpret_cast<uint64_t *>(sw + 2 * kColRows);  // [2][rows][2] sign words
    uint64_t *mbar = sbits + 4 * kColRows;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(mbar + 1);
    int *sflag = reinterpret_cast<int *>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int c = blockIdx.x, k = blockIdx.y;
    const bool dbl = mode != 3;  // double-buffered tanh rows (the squares stage two factors instead)
    const int vpr = mode == 3 ? K * (K + 1) / 2 : K;
    const size_t nrows = size_t(F.Ns) * vpr;
    const size_t r0 = nrows * c / F.rchunks, r1 = nrows * (c + 1) / F.rchunks;
    const int nbat = int((r1 - r0 + kColRows - 1) / kColRows);
    if (tid == 0) {
        mbar_init(mbar, 1);
        *sflag = 0;
    }
    if (warp == 0) tmem_alloc(tslot, tcols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    const uint32_t idesc = idesc_bf16_f32(128, MN);
    const unsigned sbo = kColRows * 16;
    const int per = MT / 4;
    auto decode = [&](size_t r, size_t &s, int &kk, int &kk2) {
        s = r / vpr;
        kk = int(r - s * vpr);
        kk2 = kk;
        if (mode == 3) {
            int a = 0;
            while (kk >= K - a) {
                kk -= K - a;
                a++;
            }
            kk2 = a + kk;
            kk = a;
        }
    };
    // batch bi: its tanh rows by cp.async (one commit group), weights and sign words
    auto stage = [&](int bi) {
        const size_t rb0 = r0 + size_t(bi) * kColRows;
        const int nb = int(min(size_t(kColRows), r1 - rb0)), sbuf = bi & 1;
        const int nf = mode == 3 ? 2 : 1;
        for (int t = tid; t < nf * nb * per; t += kColThreadsTc) {
            const int f = t / (nb * per), rem = t - f * nb * per, rr = rem / per, pc = rem - rr * per;
            size_t s;
            int kk, kk2;
            decode(rb0 + rr, s, kk, kk2);
            const size_t row = s * KK + size_t(k) * K + (f == 0 ? kk : kk2);
            const int slot = dbl ? sbuf : f;
            cp_async16_cg(sT + (size_t(slot) * kColRows + rr) * MT + 4 * pc, F.T + row * MT + 4 * pc);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        for (int rr = tid; rr < kColRows; rr += kColThreadsTc) {
            float wr = 0.f;
            uint64_t x0 = 0, x1 = 0;
            if (rr < nb) {
                size_t s;
                int kk, kk2;
                decode(rb0 + rr, s, kk, kk2);
                const size_t qo = s * KK + size_t(k) * K;
                wr = __ldg(F.B + qo + kk);
                if (mode == 0) wr *= __ldg(w + s);
                if (mode == 2) {
                    double el = 0.0;
                    for (int q = 0; q < K; q++) el += E[s * KK + q * K + q].re;
                    wr *= float(el);
                }
                x0 = F.spins[(s * K + kk) * NW];
                x1 = NW > 1 ? F.spins[(s * K + kk) * NW + 1] : 0ULL;
                if (mode == 3) {
                    wr *= (kk == kk2 ? 1.f : 2.f) * __ldg(F.B + qo + kk2);
                    x0 ^= F.spins[(s * K + kk2) * NW];
                    if (NW > 1) x1 ^= F.spins[(s * K + kk2) * NW + 1];
                }
            }
            sw[sbuf * kColRows + rr] = wr;  // 0 for rows beyond the chunk
            sbits[(sbuf * kColRows + rr) * 2] = x0;
            sbits[(sbuf * kColRows + rr) * 2 + 1] = x1;
        }
    };
    unsigned ph = 0;
    bool mma_pend = false;
    unsigned mma_ph = 0;
    if (nbat > 0) stage(0);
    if (dbl && nbat > 1) stage(1);
    const int half = tid >> 7, lt = tid & 127;  // two threads per row of A / Bt: batch rows 32 half .. +31
    for (int bi = 0; bi < nbat; bi++) {
        const int nb = int(min(size_t(kColRows), r1 - (r0 + size_t(bi) * kColRows))), sbuf = bi & 1;
        if (dbl && bi + 1 < nbat)
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        else
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();  // batch bi staged; the previous MMAs are done
        const float *t0 = sT + size_t(dbl ? sbuf : 0) * kColRows * MT, *t1 = sT + size_t(kColRows) * MT;
        const float *wb = sw + sbuf * kColRows;
        const uint64_t *bb = sbits + sbuf * kColRows * 2;
        // A: row i = lt, batch rows 32 half .. 32 half + 31
        {
            const int i = lt;
#pragma unroll 1
            for (int ro = 4 * half; ro < 4 * half + 4; ro++) {
                uint32_t wv[4];
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    uint32_t pr = 0;
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int rr = ro * 8 + h * 2 + e;
                        uint32_t val = 0;
                        if (rr < nb) {
                            if (i < N) {
                                const uint64_t x = i < 64 ? bb[2 * rr] : bb[2 * rr + 1];
                                val = ((x >> (i & 63)) & 1ULL) ? 0xBF80u : 0x3F80u;
                            } else if (i == N) {
                                val = 0x3F80u;
                            }
                        }
                        pr |= val << (16 * e);
                    }
                    wv[h] = pr;
                }
                *reinterpret_cast<uint4 *>(sA + kmajor_off(i, ro * 8, kColRows)) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
            }
        }
        // Bt: rows j = lt, lt + 128, batch rows 32 half .. 32 half + 31 (three split planes)
        for (int j = lt; j < MN; j += 128) {
#pragma unroll 1
            for (int ro = 4 * half; ro < 4 * half + 4; ro++) {
                uint32_t ph_[4], pm_[4], pl_[4];
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    ph_[h] = pm_[h] = pl_[h] = 0;
#pragma unroll
                    for (int e = 0; e < 2; e++) {
                        const int rr = ro * 8 + h * 2 + e;
                        float x = 0.f;  // rows beyond the chunk stay 0 (their tanh slots are stale)
                        if (rr >= nb) {
                        } else if (j < M) {
                            x = t0[size_t(rr) * MT + j];
                            if (mode == 3) x *= t1[size_t(rr) * MT + j];
                            x *= wb[rr];
                        } else if (j == M) {
                            x = wb[rr];
                        }
                        uint32_t a, b, d;
                        bf16_split3_trunc(x, a, b, d);
                        ph_[h] |= a << (16 * e);
                        pm_[h] |= b << (16 * e);
                        pl_[h] |= d << (16 * e);
                    }
                }
                const unsigned o = kmajor_off(j, ro * 8, kColRows);
                *reinterpret_cast<uint4 *>(sB + o) = make_uint4(ph_[0], ph_[1], ph_[2], ph_[3]);
                *reinterpret_cast<uint4 *>(sB + size_t(MN) * kColRows * 2 + o) = make_uint4(pm_[0], pm_[1], pm_[2], pm_[3]);
                *reinterpret_cast<uint4 *>(sB + size_t(2) * MN * kColRows * 2 + o) =
                    make_uint4(pl_[0], pl_[1], pl_[2], pl_[3]);
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();  // A and Bt written
        if (tid == 0) {
            tc_fence_after();
#pragma unroll 1
            for (int q = 0; q < 3; q++)
#pragma unroll 1
                for (int ks = 0; ks < kColRows / 16; ks++) {
                    const uint64_t ad = smem_desc(sA + ks * 256, 128, sbo);
                    const uint64_t bd = smem_desc(sB + size_t(q) * MN * kColRows * 2 + ks * 256, 128, sbo);
                    mma_bf16(tbase, ad, bd, idesc, bi > 0 || q > 0 || ks > 0);
                }
            mma_commit(mbar);
        }
        if (!dbl && bi + 1 < nbat) stage(bi + 1);  // the single tanh buffer is free after the build
        const bool done = mbar_wait(mbar, ph);      // A and Bt are read by the MMAs
        if (!done) {
            *sflag = 1;
            if (tid == 0) {
                mma_pend = true;
                mma_ph = ph;
            }
        }
        ph ^= 1;
        __syncthreads();
        if (*sflag) break;
        if (dbl && bi + 2 < nbat) stage(bi + 2);  // buffer bi & 1 was consumed by the build
    }
    if (!*sflag && nbat > 0) {
        if (warp < 4) {
            tc_fence_after();
            // the chunk's partial: thread i of warps 0-3 holds row i
            const int i = tid;
            float *o = out + size_t(c) * P + size_t(k) * L;
            for (int c0 = 0; c0 < MN; c0 += 16) {
                float dv[16];
                tmem_ld16(tbase + (uint32_t(32 * warp) << 16) + uint32_t(c0), dv);
#pragma unroll
                for (int q = 0; q < 16; q++) {
                    const int j = c0 + q;
                    if (i < N && j < M)
                        o[N + M + size_t(i) * M + j] = dv[q];
                    else if (i < N && j == M)
                        o[i] = dv[q];
                    else if (i == N && j < M)
                        o[N + j] = dv[q];
                }
            }
        }
    } else if (nbat == 0) {
        float *o = out + size_t(c) * P + size_t(k) * L;  // an empty chunk contributes zeros
        for (int t = tid; t < L; t += kColThreadsTc) o[t] = 0.f;
    }
    if (tid == 0 && *sflag) {
        atomicOr(err, kErrTimeout);
        if (mma_pend) mbar_wait(mbar, mma_ph);
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tbase, tcols);
}

}  // namespace

bool rows_tc_fits(const FactArgs &F) {
    if (F.N + 1 > 144 || F.M + 1 > 256) return false;
    const RowsTcShape s = rows_tc_shape(F);
    return s.abytes + s.bbytes + 64 + 512 <= size_t(227) * 1024;
}

size_t rows_tc_image_elems(const FactArgs &F) {
    return size_t(F.K) * 3 * round16(F.M + 1) * round16(F.N + 1);
}

cudaError_t prepare_frows_tc(const FactArgs &F) {
    if (!rows_tc_fits(F)) return cudaSuccess;
    const RowsTcShape s = rows_tc_shape(F);
    return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_frows_tc));
}

cudaError_t launch_frows_tc(const FactArgs &F, const float *v, float *u, int *err, cudaStream_t st) {
    const RowsTcShape s = rows_tc_shape(F);
    const size_t n = rows_tc_image_elems(F) / 3;
    k_rows_bimg<<<int(std::min<size_t>((n + 255) / 256, 1024)), 256, 0, st>>>(F, s.NP, s.MN, v, F.tcimg);
    int dev = 0, sms = 148, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_frows_tc, kTcThreads, s.smem);
    const int ntiles = (F.Ns + kTcThreads / F.K - 1) / (kTcThreads / F.K);
    const int grid = std::max(1, std::min(ntiles, sms * std::max(per_sm, 1)));
    k_frows_tc<<<grid, kTcThreads, s.smem, st>>>(F, s.NP, s.MN, s.tcols, s.abytes, s.bbytes, F.tcimg, u, err);
    return cudaGetLastError();
}

}  // namespace nqes

namespace nqes {

bool cols_tc_fits(const FactArgs &F) {
    if (F.N + 1 > 128 || F.M + 1 > 256) return false;
    const ColsTcShape s = cols_tc_shape(F);
    return s.tbytes + s.abytes + s.bbytes + 2 * kColRows * 20 + 64 <= size_t(227) * 1024;
}

cudaError_t prepare_fcols_tc() { return allow_max_dynamic_smem(reinterpret_cast<const void *>(k_fcols_tc)); }

cudaError_t launch_fcols_tc(const FactArgs &F, int mode, const float *w, const cplx *E, float *out, int *err,
                            cudaStream_t st) {
    const ColsTcShape s = cols_tc_shape(F);
    dim3 g(F.rchunks, F.K);
    k_fcols_tc<<<g, kColThreadsTc, s.smem, st>>>(F, mode, s.MN, s.tcols, s.tbytes, s.abytes, s.bbytes, w, E, out, err);
    return cudaGetLastError();
}

}  // namespace nqes
