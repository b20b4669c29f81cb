// Internal interfaces between the host orchestration (nqes_api.cu) and the
// kernel translation units. Not part of the public C ABI.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "nqes_math.cuh"

namespace nqes {

// Per-SR-step scalars. Lives in device memory so that one captured CUDA graph
// serves every step: the host rewrites it before each launch.
struct StepParams {
    uint64_t seed;      // chain c uses pcg64(seed + c)
    double lr;          // learning rate for w -= lr * x
    double reglam;      // lambda of S + lambda diag(S)
    double rtol;        // MINRES-QLP relative tolerance
    uint64_t maxit;     // MINRES-QLP iteration limit (already capped)
};

// Device tables derived from the weights at the start of every SR step.
// Layouts: ch/sh [kk][i][j] = cosh(2 w), sinh(2 w); eup/edn [kk][i] =
// exp(-2 a) (flip of an up spin) and exp(+2 a) (flip of a down spin).
template <class S> struct Tables {
    const S *ch, *sh, *eup, *edn;
};

struct Shape {
    int N, M, K, L, P, NW;
};

template <class S> struct SampleArgs {
    Shape sh;
    int chains, m, burn;
    int tk;                     // threads per RBM column block (multiple of 32)
    const StepParams *sp;
    Tables<S> tab;
    const cplx *a, *b, *w;      // weights, reference layout
    const double *J;            // N×N row-major
    double h;
    // Local energy: ham 0, H = sum_{i>j} J_ij sz_i sz_j - h sum_i sx_i (the
    // ising-like models); ham 1, H = sum_{i>j} J_ij (sx_i sx_j + sy_i sy_j +
    // delta sz_i sz_j) (the Heisenberg-like models hs and xxz).
    int ham;
    double delta;
    S *O;                       // Ns × P log-derivatives (row s = c*m + t)
    cplx *E;                    // Ns × K² local-energy matrices
    uint64_t *spins;            // Ns × K × NW configurations
    unsigned long long *accepted;  // per chain
    int *err;                   // error bits (see kErr*)
    // Evaluation mode (configs given, no sampling): when cfg != nullptr the
    // kernel evaluates Phi / tanh(theta) / E / O at cfg[c] for c < chains.
    const uint64_t *cfg;
    cplx *phi_out, *tanh_out;   // chains × K², chains × M × K² (optional)
    cplx *dm_out;               // chains × K²: E = Phi^-1 (D o Phi)'s D (optional)
    // Correlation mode (corr != nullptr): per-chain sums of the x, z, xx, zz
    // observables instead of E and O; layout per chain [x N×K²][z N×K²]
    // [xx N×N×K²][zz N×N×K²] (corr_stride scalars), scratch N×N×K² per chain.
    S *corr, *corr_scratch;
    size_t corr_stride;
    // Rejection filter (real arithmetic only; nullptr = off): FP32 roundings
    // of the FP64 tables cosh(2w), sinh(2w), exp(-2a), exp(2a).
    const float *c32, *s32, *eu32, *ed32;
};

template <class S> cudaError_t launch_corr_reduce(const S *acc, int chains, size_t stride, S *out, cudaStream_t st);
// E (pseudo-inverse) and O (zero) at the evaluated configurations whose Phi is
// rank deficient; O rows of o_doubles doubles.
cudaError_t launch_eval_singular(int count, int K, const cplx *phi, const cplx *dm, cplx *E, double *O,
                                 size_t o_doubles, cudaStream_t st);

// Mixed-precision sampler (real weights): FP32 factors, products and accept
// decisions with a certified error bound, FP64 shadow of theta, exact FP64
// Phi after every sweep, exact FP64 decision when the bound is inconclusive.
// x / d by one high multiply for 32-bit x < 2^32 / d: with m = ceil(2^32 / d)
// and e = m d - 2^32 < d, x m / 2^32 = x / d + x e / (d 2^32) and the second
// term stays below 1/d, so the floor is exact (d = 1: x itself). Integer
// divisions by a run-time divisor cost tens of instructions; the index math
// of the factored passes' staging and epilogues uses this instead.
struct FastDiv {
    unsigned d, m;
};
__host__ __device__ inline FastDiv fast_div(unsigned d) {
    FastDiv f;
    f.d = d;
    f.m = d <= 1 ? 0u : unsigned((0x100000000ULL + d - 1) / d);
    return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned x, FastDiv f) { return f.d <= 1 ? x : __umulhi(x, f.m); }

struct MixedArgs {
    Shape sh;
    int chains, m, burn, tk;
    const StepParams *sp;
    const float *ch, *sh32, *eup, *edn;  // FP32 cosh(2w), sinh(2w) [kk][i][j]; exp(-2a), exp(2a) [kk][i]
    const double *w64, *a64, *b64;       // real weights [kk][i][j], [kk][i], [kk][j]
    const double *J;
    double h;
    float *FT, *FB;                      // factors of O (kernels_factored.cu): FT Ns×K×K×fact_mt(M), FB Ns×K×K
    cplx *E;                             // Ns × K² local-energy matrices (FP64)
    uint64_t *spins;
    unsigned long long *accepted;        // per chain
    unsigned long long *exact;           // per chain: decisions taken by the exact FP64 path
    int *err;
    int exact_all;                       // 1: every decision through the exact FP64 path (test hook)
    // Decision-warp form (kernels_sample_warp.cu): G lanes per RBM, U units per
    // lane, tables padded to MP = G*U units per (kk, i) row: FP32 cosh(2w),
    // sinh(2w) and w as hi + lo [kk][i][MP]; b as hi + lo [kk][MP].
    const float *cp, *spp, *whp, *wlp, *bh, *bl;
    const float *cpl, *spl;              // the roundings' remainders: cosh(2w) - cp, sinh(2w) - spp [kk][i][MP]
    const float *bnd;                    // per (kk, i): float4 bound record, then per kk 2 max_j sum_i |w_ij|
    const double *etab;                  // e^{-n/64}, n < kExpTabN (nqes_math.cuh exp_neg_tab)
    FastDiv fdN, fdM, fdMP, fdMT;        // the divisors N, M, MP and fact_mt(M) of the index math
    int G, U, MP;
    int stage;                           // 1: bulk-copy cp, spp, whp, wlp into shared memory first
    int stage_fault;                     // test hook (NQES_OPT_TEST_STAGE_WAIT): the staging wait runs out
    // FP64 outputs (NQES_PRECISION_CERTIFIED): E from FP64 flip ratios and the
    // dense FP64 O (P per sample) instead of the FP32 factors
    int out64;
    double *O64;
    int o_split;  // out64: each entry of O64 stored as its double-float split (hi, lo) for the fused S·v
    const double *c64, *s64, *eup64, *edn64;  // FP64 tables [kk][i][j], [kk][i]
    // FP64 local energies with the FP32 factor outputs (MIXED, NQES_OPT_MIXED_ENERGY64):
    // the flip ratios as double-float products over (cp + cpl, spp + spl) on
    // the FP32 pipe with tanh of the exact theta in FP64 (1) or from its FP32
    // value and the low part of theta (2); O as factors; 0: FP32 ratios
    int e64;
};
size_t mixed_smem_bytes(const Shape &sh);
int dw_units(const Shape &sh, int *G_out);  // U of the decision-warp form, 0 if it does not apply
size_t dw_smem_bytes(const Shape &sh, int MP, bool staged, bool out64 = false);
cudaError_t prepare_sample_dw(const Shape &sh, int MP);
cudaError_t launch_sample_dw(const MixedArgs &a, int warps, cudaStream_t st);
cudaError_t launch_exp_table(double *tab, cudaStream_t st);  // tab[n] = e^{-n/64}, n < kExpTabN
cudaError_t dw_occupancy(const Shape &sh, int threads, size_t smem, int *blocks_per_sm);
cudaError_t launch_tables_dw(const Shape &sh, int MP, const cplx *b, const cplx *w, float *cp, float *spp, float *whp,
                             float *wlp, float *bh, float *bl, float *bnd, float *cpl, float *spl, cudaStream_t st);
cudaError_t prepare_sample_mixed(const Shape &sh);
cudaError_t launch_sample_mixed(const MixedArgs &a, cudaStream_t st);
cudaError_t launch_tables_mixed(const Shape &sh, const cplx *a, const cplx *b, const cplx *w, float *ch, float *sh32,
                                float *eup, float *edn, double *w64, double *a64, double *b64, cudaStream_t st);

enum : int {
    kErrNonFinite = 1,      // a non-finite amplitude ratio, energy or derivative
    kErrSingular = 2,       // a sample was taken at a singular Phi
    kErrMinresNonFinite = 4,
    kErrMinresCap = 8,      // MINRES-QLP stopped at the device-side iteration cap
    kErrTimeout = 16,       // a bounded device-side wait ran out
    kErrLaunch = 32,        // a kernel got less dynamic shared memory than its layout needs
};

// True when the launch's dynamic shared memory holds `need` bytes. Kernels
// that carve their dynamic shared memory check this at entry (uniformly over
// the block) and return with kErrLaunch instead of addressing past the
// allocation, should a host-side size ever disagree with the device layout.
__device__ __forceinline__ bool dyn_smem_covers(size_t need) {
    unsigned have;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(have));
    return need <= size_t(have);
}

size_t sample_smem_bytes(const Shape &sh, int threads, bool complex_arith);
int sample_threads(int K, int tk);  // K*tk threads per chain
template <class S> cudaError_t launch_sample(const SampleArgs<S> &a, int threads, cudaStream_t st);
template <class S> cudaError_t launch_tables(const Shape &sh, const cplx *a, const cplx *w, S *ch, S *shh, S *eup,
                                             S *edn, cudaStream_t st);

// ---- moments, S·v, MINRES-QLP ----

// Device-resident MINRES-QLP scalar state (double-buffered by the host
// schedule; see kernels_solve.cu).
struct QlpState {
    // recurrence scalars (code/minresqlp.h:128-138 names)
    double beta, tau, taul, phi, betan, gmin, gminl;
    double cs, sn, cr1, sr1, cr2, sr2, dltan, eplnn;
    double gama, gamal, gamal2, eta, etal, etal2;
    double vepln, veplnl, veplnl2, ul3, ul2, ul, u;
    double gama_qlp, gamal_qlp, vepln_qlp, u_qlp, ul_qlp;
    double rnorm, xnorm, xl2norm, axnorm, anorm, acond, relres, beta1;
    // per-iteration values consumed by the vector kernel
    double alfa, epln, dlta_qlp, gama_tmp, gamal3, veplnl2_v, etal_v;
    double w_gamal_qlp, w_vepln_qlp, w_gama_qlp, w_ul_qlp, w_u_qlp;
    double cr2_v, sr2_v;   // P_{k-2,k} rotation as of the vector update
    unsigned long long iters, qlp_iters, cap, iters_snapshot;
    unsigned long long bodies;  // executions of the loop body (for launch counts)
    int flag;
    int mode;         // 0: no update, 1: MINRES update, 2: QLP update, 3: x = b/alfa
    int qlp_first;    // QLP update is the first one (rebuild w's)
    int running;
};

// Lanczos-side scalars of MINRES-QLP. The Lanczos chain of step j (S v_j,
// r3, the next v) runs beside the QLP chain of step j - 1, so the scalars the
// QLP chain reads live in slots: beta_j at beta[j % 3], alfa_j and |r3_j|^2
// (= beta_{j+1}^2) at alfa[j % 2] and bn2[j % 2]. j is the step whose v the
// next S·v multiplies; arrived counts the blocks of the kernel that advances it.
struct LzState {
    double beta[3];
    double alfa[2], bn2[2];
    unsigned long long j;
    unsigned int arrived;
};

// Reduction partial buffers: one slot per 64-element MINRES-QLP vector block.
// P <= 4 * (128 + 512 + 128*512) gives at most 4136 blocks; three regions of
// this stride live in SolveBufs::part (alfa, |r3|^2, |b|^2) and one in ovpart.
constexpr int kPartStride = 4160;

template <class S> cudaError_t prepare_sample(const Shape &sh);

// Factors of O in the mixed form (kernels_factored.cu): for sample s,
// T[s][k][kk][j] = tanh theta_j of configuration kk under RBM k (rows padded
// with zeros to MT = fact_mt(M) floats) and B[s][k][kk] =
// (Phi^-1)_{k,kk} Phi_{kk,k}; the spins give the signs.
struct FactArgs {
    int N, M, K, NW, Ns, rchunks, MT;
    int ic;  // rows of W staged per chunk by the rows pass (set at launch)
    const float *T, *B;
    const uint64_t *spins;
    int tc;            // rows pass on the tensor cores (kernels_factored_tc.cu)
    int tcc;           // column passes (S·v and moments) on the tensor cores
    uint16_t *tcimg;   // its BF16 split image of the parameter vector
    int *err;
    const int *guard;  // see loop_guard_off (nullptr: no guard)
};
__host__ __device__ inline int fact_mt(int M) { return (M + 3) & ~3; }

// A solve's factored S·v passes as a member of a grouped launch (a batch's
// loop body): its factors, v (FP32 mirror), u = O v and the O^T u partials.
struct FactMember {
    FactArgs F;  // F.ic set as its own rows pass would
    const float *v32;
    float *u32, *ypart32;
    int gn, zg;  // column pass: i groups per row set and i blocks
};
// Kernel variants, shared memory and blocks of a solve's rows and column
// passes; solves of one variant can share a launch (the launch takes the
// largest shared memory of its solves).
struct FactGroupPlan {
    int rows_variant, rows_blocks, ic;
    size_t rows_smem;
    int cols_variant, cols_blocks, gn, zg;
    size_t cols_smem;
};
FactGroupPlan fact_group_plan(const FactArgs &F);
// Blocks, shared memory and staged rows (ic) of the rows pass in `variant`;
// variant 6 is variant 2 (M <= 64) with 4 rows a thread group instead of 2
// (fewer blocks, more work a block: the form for a large group), with the
// same arithmetic per row.
void fact_rows_geometry(int variant, const FactArgs &F, int *blocks, size_t *smem, int *ic);
cudaError_t prepare_fact_group(const FactGroupPlan &g);  // outside stream capture
cudaError_t launch_frows_group(int variant, const FactMember *tab, const int *first, int n, int blocks, size_t smem,
                               cudaStream_t st);
cudaError_t launch_fcols_group(int variant, const FactMember *tab, const int *first, int n, int blocks, size_t smem,
                               cudaStream_t st);

// Solve m of a grouped launch owns blocks first[m] .. first[m + 1] - 1.
__device__ __forceinline__ int group_member(const int *__restrict__ first, int n, int b) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(first + mid) <= b)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Lets kernel `fn` take as much dynamic shared memory as the device allows.
// The limit is a per-kernel global: set to one context's need, it would cap
// the same kernel launched (or replayed from a captured graph) by a context of
// a larger shape, so it is only ever raised, to the device maximum.
inline cudaError_t allow_max_dynamic_smem(const void *fn) {
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa{};
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, fn);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - int(fa.sharedSizeBytes));
    return e;
}
bool rows_tc_fits(const FactArgs &F);
size_t rows_tc_image_elems(const FactArgs &F);
cudaError_t prepare_frows_tc(const FactArgs &F);
cudaError_t launch_frows_tc(const FactArgs &F, const float *v, float *u, int *err, cudaStream_t st);
bool cols_tc_fits(const FactArgs &F);
cudaError_t prepare_fcols_tc();
cudaError_t launch_fcols_tc(const FactArgs &F, int mode, const float *w, const cplx *E, float *out, int *err,
                            cudaStream_t st);
cudaError_t prepare_frows(const FactArgs &F);
cudaError_t launch_frows(const FactArgs &F, const float *v, float *u, cudaStream_t st);
cudaError_t launch_fcols(const FactArgs &F, const float *w, float *ypart, cudaStream_t st);
cudaError_t launch_fmoments(const FactArgs &F, const cplx *E, float *po, float *pf, float *ps2, cudaStream_t st);
cudaError_t launch_fmoment_final(const FactArgs &F, const StepParams *sp, const float *po, const float *pf,
                                 const float *ps2, const cplx *eloc, double *o, double *skk, double *f, int *err,
                                 cudaStream_t st);
cudaError_t launch_fO(const FactArgs &F, int first, int count, float *O, cudaStream_t st);

template <class S> struct SolveBufs {
    Shape sh;
    int Ns;
    const S *O;
    const cplx *E;       // per-sample E matrices (for eloc and e_mat)
    S *o, *skk, *f;      // moments (P)
    S *u;                // Ns: O v
    S *ypart;            // rchunks × P partial O^H u
    int rchunks;
    S *r1, *r2, *r3, *v, *w, *wl, *wl2, *x, *xl2;
    S *vq;               // v_j for the QLP chain at vq + (j % 3) P (written two
                         // loop bodies before the QLP step that reads it)
    double *part;        // reduction partials (>= 2 * 1024)
    S *ovpart;           // partial o·v
    QlpState *qs;
    LzState *lz;
    const StepParams *sp;
    cplx *emat;          // K² mean E (unnormalised by N)
    cplx *eloc;          // mean trace
    int *err;
    cudaGraphConditionalHandle cond;
    int use_cond;
    // Loop-body guard of a batched solve (nullptr outside a batch): the
    // MINRES-QLP loop of a batch runs until every member has stopped, and a
    // member's loop-body kernels return at entry once *guard (its
    // QlpState::running) is 0. Its own loop condition is then left alone
    // (use_cond 0): one kernel after all members' bodies sets the batch's.
    const int *guard;
    // Partials of O^H u that the Lanczos epilogue sums over (sv_colsum):
    // svp rows of P at ysv. The two-pass S·v writes rchunks rows to ypart; the
    // fused S·v (fG > 0: real arithmetic, kernels_sv_fused.cu) one row per CTA.
    int svp;
    S *ysv;
    int fG, fNB;  // fused S·v: rows per staged group and groups in its ring
    // O stored as double-float (hi, lo) pairs in its FP64 slots (the certified
    // sampler writes it so when the fused S·v runs): the fused S·v and the
    // moments read the pairs directly
    int o_split;
    // Mixed precision (real arithmetic only, fact = 1): O held as its factors
    // and the two passes of S·v and the moments computed from them in FP32
    // (kernels_factored.cu); v is mirrored into v32 by the kernels that
    // produce it; ypart32 holds rchunks × P partials (3 × for the moments).
    int fact;
    FactArgs F;
    float *v32, *u32, *ypart32;
};

// Pair-interleaved double-float rows: per pair of entries (2q, 2q + 1) the 16
// bytes (hi_2q, hi_2q+1, lo_2q, lo_2q+1), so that one 16-byte load gives both
// entries' hi and lo parts as packed FP32 pairs (nqes_math.cuh f2_*). Float
// index of entry p's hi part within its row; its lo part is two floats further.
__host__ __device__ inline size_t dfpair_hi(size_t p) { return 4 * (p >> 1) + (p & 1); }

// Fused S·v over the dense FP64 O (kernels_sv_fused.cu): one read of O,
// double-float arithmetic on the FP32 pipe. sv_fused_plan gives the rows per
// staged group and the CTAs (false: the shape needs the two-pass S·v).
bool sv_fused_plan(int Ns, int P, int *G_out, int *NB_out, int *ctas_out);
cudaError_t prepare_sv_fused(int P);
cudaError_t launch_sv_fused(int Ns, int P, int G, int NB, int ctas, const double *O, const double *v, double *ypart,
                            int *err, const int *guard, cudaStream_t st, bool o_split = false);

// Sets the batched MINRES-QLP loop's condition: 1 while any member's flag
// (its QlpState::running) is set.
cudaError_t launch_batch_cond(const int *const *flags, int n, cudaGraphConditionalHandle cond, cudaStream_t st);

// True, uniformly over the block, when a loop-body guard is set and its flag
// is 0: the kernel then returns at entry (every thread of the block, before
// any barrier). The flag is read once by thread 0: in the loop body where the
// member's solve stops, the QLP kernel beside may clear it while blocks of a
// Lanczos kernel start, and the Lanczos step of that body is never used.
__device__ __forceinline__ bool loop_guard_off(const int *guard) {
    if (!guard) return false;
    __shared__ int s_guard;
    if (threadIdx.x == 0) s_guard = *reinterpret_cast<const volatile int *>(guard);
    __syncthreads();
    return s_guard == 0;
}

template <class S> cudaError_t launch_moments(const SolveBufs<S> &b, cudaStream_t st);
template <class S> cudaError_t launch_minres_init(const SolveBufs<S> &b, cudaStream_t st);
// One MINRES-QLP iteration as two chains: the Lanczos step (S v_j, r3,
// v_{j+1}) and the QLP step of the previous iteration (scalar recurrence, w
// and x updates); launch_minres_init also runs the first Lanczos step.
template <class S> cudaError_t launch_lanczos_step(const SolveBufs<S> &b, cudaStream_t st);
template <class S> cudaError_t launch_qlp_step(const SolveBufs<S> &b, cudaStream_t st);
template <class S> cudaError_t launch_apply_S(const SolveBufs<S> &b, const S *v, S *out, cudaStream_t st);
// The MINRES-QLP vector kernels of a group of solves (a batch's loop body), one
// launch per kernel: tab (device memory) holds the solves' buffers, first[m] the
// first block of solve m (first[0] = 0, first[n] = blocks), each solve taking
// minres_vector_blocks(P) blocks. The Lanczos part (r3, alfa, beta, v_{j+1})
// follows the group's S·v passes; the QLP part runs beside it.
int minres_vector_blocks(int P);
template <class S>
cudaError_t launch_lanczos_group(const SolveBufs<S> *tab, const int *first, int n, int blocks, cudaStream_t st);
template <class S>
cudaError_t launch_qlp_group(const SolveBufs<S> *tab, const int *first, int n, int blocks, cudaStream_t st);
template <class S> cudaError_t launch_sv_rows_only(const SolveBufs<S> &b, cudaStream_t st);
template <class S> cudaError_t launch_sv_cols_only(const SolveBufs<S> &b, cudaStream_t st);
template <class S> cudaError_t launch_sv_only(const SolveBufs<S> &b, cudaStream_t st);  // the step's S·v passes
template <class S> cudaError_t launch_moment_part_only(const SolveBufs<S> &b, cudaStream_t st);
template <class S> cudaError_t launch_update(const Shape &sh, const StepParams *sp, const S *x, cplx *a, cplx *b,
                                             cplx *w, cudaStream_t st);

}  // namespace nqes
