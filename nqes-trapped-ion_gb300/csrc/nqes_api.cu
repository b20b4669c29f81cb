// Host side of libnqes: the C ABI of include/nqes.h.
//
// One SR step (code/rbm.cc:564-719) is one CUDA graph launch:
//   [clear error word] -> tables(w) -> sampler (one CTA per chain) ->
//   moments -> MINRES-QLP init -> while (running) { S·v rows, S·v cols,
//   Lanczos a, Lanczos b, QLP scalars, QLP vectors } -> w -= lr x
// The while loop is a graph conditional node whose condition the QLP scalar
// kernel sets, so the Krylov solve runs without host round trips. Per-step
// scalars (seed, lr, reglam, rtol, maxit) live in device memory and are
// rewritten before each launch; the graph is rebuilt only when the chain
// count, samples per chain, burn-in, arithmetic or thread shape change.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <type_traits>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/nqes.h"
#include "nqes_internal.h"
#include "pcg64.cuh"

using namespace nqes;

namespace {
// NVTX range over a host-side phase of an SR step (visible in Nsight Systems:
// argument checks and buffer sizing, graph capture, the graph launch, the
// result read-back). The device phases inside a step run in one CUDA graph.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
}  // namespace

struct nqes_ctx {
    Shape sh{};
    int device = 0;
    cudaStream_t st = nullptr;
    cudaStream_t st_qlp = nullptr;                       // the QLP chain's capture stream
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  // its fork from / join to st in the loop body
    double h = 0;
    int arith_opt = NQES_ARITH_AUTO;
    int precision = NQES_PRECISION_FP64;
    // mixed-precision tables: FP32 cosh/sinh(2w), exp(-+2a); FP64 real w, a, b
    float *mch = nullptr, *msh = nullptr, *meup = nullptr, *medn = nullptr;
    double *mw = nullptr, *ma = nullptr, *mb = nullptr;
    unsigned long long *exact = nullptr;           // per chain
    // decision-warp form of the mixed sampler (dw_U = 0: block form)
    int dw_G = 0, dw_U = 0, dw_MP = 0;
    float *dcp = nullptr, *dsp = nullptr, *dwh = nullptr, *dwl = nullptr, *dbh = nullptr, *dbl = nullptr;
    float *dcpl = nullptr, *dspl = nullptr;  // remainders of the FP32 cosh / sinh tables (double-float ratios)
    float *dbnd = nullptr;  // K·N float4 bound records, then K row-sum maxima
    double *etab = nullptr; // e^{-n/64} for the row rebuilds (exp_neg_tab)
    float *v32 = nullptr, *u32 = nullptr, *ypart32 = nullptr;
    uint16_t *tcimg = nullptr;  // BF16 split image of v for the tensor-core rows pass
    int tensor_cores = 1;       // NQES_OPT_TENSOR_CORES: 0 off, 1 where it pays off, 2 wherever it fits
    int ham = NQES_HAM_ISING_LIKE;  // local-energy form (nqes_set_hamiltonian)
    double ham_delta = 0.0;
    int step_precision = NQES_PRECISION_FP64;      // precision of the allocated step buffers
    int tk_opt = 0;
    uint64_t minres_cap = 100000;
    bool reject_filter = false;  // FP32 rejection filter in the FP64 real sampler (opt-in)
    // autotuner (NQES_OPT_AUTOTUNE): launch shape of the sampler chosen by timing,
    // valid for tune_key = (chains, samples, burn-in, precision, arith)
    bool autotune = false;
    long long tune_key[5] = {-1, -1, -1, -1, -1};
    int tk_tuned = 0, dw_force_warps = 0, dw_force_stage = 0;
    // Chains the sampler's launch shape is planned for (0: the step's own).
    // A batch sets it to the chains of all its members while it builds its
    // graph: the members' samplers then share the GPU.
    int plan_chains = 0;
    int stage_fault = 0;  // NQES_OPT_TEST_STAGE_WAIT
    int mixed_e64 = 2;  // NQES_OPT_MIXED_ENERGY64: 0, 1 or 2
    bool mixed_exact_all = false;  // MIXED: every decision through the exact FP64 path
    bool weights_real = true;
    std::string err;

    cplx *a = nullptr, *b = nullptr, *w = nullptr;
    double *J = nullptr;
    void *tab = nullptr;  // ch, sh (K·N·M each), eup, edn (K·N each), sized for complex
    StepParams *sp = nullptr, *sp_host = nullptr;
    QlpState *qs = nullptr, *qs_host = nullptr;
    LzState *lz = nullptr;
    int *err_d = nullptr, *err_host = nullptr;
    cplx *emat_d = nullptr, *eloc_d = nullptr, *emat_host = nullptr;

    // per-shape step buffers
    int chains = 0, m = 0, arith = 0;
    size_t Ns = 0;
    void *O = nullptr;
    cplx *E = nullptr;
    uint64_t *spins = nullptr;
    unsigned long long *accepted = nullptr;
    void *u = nullptr, *ypart = nullptr, *vecs = nullptr, *ovpart = nullptr;
    double *part = nullptr;
    int rchunks = 1;
    // fused S·v over the dense FP64 O (real arithmetic): rows per staged
    // group, CTAs and their partials (fG = 0: the two-pass S·v)
    int fG = 0, fNB = 0, fctas = 0;
    double *ysv = nullptr;
    int fused_opt = -1, step_fused_opt = -1;  // NQES_OPT_FUSED_SV, and its value when the buffers were sized

    // Generation of the step buffers: bumped whenever they are freed or
    // reallocated, so that a batch graph that baked in the old addresses is
    // never replayed on new ones.
    uint64_t buf_gen = 0;

    cudaGraphExec_t exec = nullptr;
    int g_chains = -1, g_m = -1, g_burn = -1, g_arith = -1, g_tk = -1, g_prec = -1;
    bool have_step = false;
    int last_burn = 0, last_tk = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

// Error text for calls that have no context (reported by nqes_last_error(NULL)),
// per calling thread: the serving loop's workers create contexts concurrently.
thread_local std::string g_create_error;

namespace nqes {
void set_global_error(const std::string &msg) { g_create_error = msg; }
}  // namespace nqes

#define NQES_CUDA(call)                                                                                   \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) {                                                                          \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                                \
            return e_ == cudaErrorMemoryAllocation ? NQES_ERR_OOM : NQES_ERR_CUDA;                        \
        }                                                                                                 \
    } while (0)

namespace {

template <class T> int dalloc(nqes_ctx *ctx, T **p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
    if (e != cudaSuccess) {
        ctx->err = "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes: " + cudaGetErrorString(e);
        return NQES_ERR_OOM;
    }
    return NQES_OK;
}
template <class T> void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

size_t ssize(int arith) { return arith == NQES_ARITH_COMPLEX ? sizeof(cplx) : sizeof(double); }

void free_step_buffers(nqes_ctx *ctx) {
    dfree(ctx->O);
    dfree(ctx->E);
    dfree(ctx->spins);
    dfree(ctx->accepted);
    dfree(ctx->u);
    dfree(ctx->ypart);
    dfree(ctx->vecs);
    dfree(ctx->ovpart);
    dfree(ctx->part);
    dfree(ctx->exact);
    dfree(ctx->v32);
    dfree(ctx->u32);
    dfree(ctx->ypart32);
    dfree(ctx->tcimg);
    dfree(ctx->ysv);
    ctx->fG = ctx->fNB = ctx->fctas = 0;
    if (ctx->exec) cudaGraphExecDestroy(ctx->exec);
    ctx->exec = nullptr;
    ctx->g_chains = -1;
    ctx->buf_gen++;
    ctx->chains = ctx->m = 0;
    ctx->Ns = 0;
    ctx->have_step = false;
}

int ensure_step_buffers(nqes_ctx *ctx, int chains, int m, int arith) {
    if (ctx->chains == chains && ctx->m == m && ctx->arith == arith && ctx->step_precision == ctx->precision &&
        ctx->step_fused_opt == ctx->fused_opt && ctx->O)
        return NQES_OK;
    free_step_buffers(ctx);
    const Shape &sh = ctx->sh;
    const size_t Ns = size_t(chains) * m, P = size_t(sh.P), ss = ssize(arith);
    const int nb = int((P + 255) / 256);
    const int ctiles = nb;
    ctx->rchunks = std::max(1, std::min(32, int((Ns + 255) / 256)));
    ctx->rchunks = std::max(1, std::min(ctx->rchunks, std::max(1, 600 / std::max(1, ctiles))));
    int rc;
    const bool mixed = ctx->precision == NQES_PRECISION_MIXED;
    if (mixed) {
        // O as its factors (K^2 (M + 1) floats per sample); column sums over
        // chunks of ~128 samples, 3 partial sets for the moments; at most 256
        // chunks, a multiple of 2 SMs / K when that many: the column pass (2
        // CTAs per SM, one per chunk and state) then fills whole waves
        ctx->rchunks = int(std::max<size_t>(1, std::min<size_t>(256, (Ns + 127) / 128)));
        {
            int sms = 148;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
            const int q = std::max(1, 2 * sms / sh.K);
            if (ctx->rchunks >= q) ctx->rchunks = ctx->rchunks / q * q;
        }
        const size_t KK = size_t(sh.K) * sh.K;
        if ((rc = dalloc(ctx, reinterpret_cast<unsigned char **>(&ctx->O), Ns * KK * (fact_mt(sh.M) + 1) * sizeof(float))) ||
            (rc = dalloc(ctx, &ctx->exact, size_t(chains))) || (rc = dalloc(ctx, &ctx->v32, P)) ||
            (rc = dalloc(ctx, &ctx->u32, Ns)) || (rc = dalloc(ctx, &ctx->ypart32, 3 * size_t(ctx->rchunks) * P)))
            return rc;
        FactArgs F{};
        F.N = sh.N;
        F.M = sh.M;
        F.K = sh.K;
        if ((rc = dalloc(ctx, &ctx->tcimg, rows_tc_image_elems(F)))) return rc;
    } else if ((rc = dalloc(ctx, reinterpret_cast<unsigned char **>(&ctx->O), Ns * P * ss))) {
        return rc;
    } else if (ctx->precision == NQES_PRECISION_CERTIFIED && (rc = dalloc(ctx, &ctx->exact, size_t(chains)))) {
        return rc;
    }
    ctx->step_precision = ctx->precision;
    ctx->step_fused_opt = ctx->fused_opt;
    // the fused S·v: by default in the certified form (FP64-grade results);
    // the FP64 form keeps IEEE FP64 arithmetic unless asked
    const bool fused = ctx->fused_opt < 0 ? ctx->precision == NQES_PRECISION_CERTIFIED : ctx->fused_opt == 1;
    if (!mixed && arith == NQES_ARITH_REAL && fused && sv_fused_plan(int(Ns), sh.P, &ctx->fG, &ctx->fNB, &ctx->fctas)) {
        if ((rc = dalloc(ctx, &ctx->ysv, size_t(ctx->fctas) * P))) return rc;
        const cudaError_t e = prepare_sv_fused(sh.P);
        if (e != cudaSuccess) {
            ctx->err = std::string("fused S·v attributes: ") + cudaGetErrorString(e);
            return NQES_ERR_CUDA;
        }
    } else {
        ctx->fG = ctx->fNB = ctx->fctas = 0;
    }
    if ((rc = dalloc(ctx, &ctx->E, Ns * sh.K * sh.K))) return rc;
    if ((rc = dalloc(ctx, &ctx->spins, Ns * sh.K * sh.NW))) return rc;
    if ((rc = dalloc(ctx, &ctx->accepted, size_t(chains)))) return rc;
    if ((rc = dalloc(ctx, reinterpret_cast<unsigned char **>(&ctx->u), Ns * ss))) return rc;
    // ypart doubles as scratch for the moment partials: 3 × rchunks × P scalars
    // (the mixed form keeps its partials in ypart32)
    if ((rc = dalloc(ctx, reinterpret_cast<unsigned char **>(&ctx->ypart), mixed ? 1 : 3 * size_t(ctx->rchunks) * P * ss)))
        return rc;
    if ((rc = dalloc(ctx, reinterpret_cast<unsigned char **>(&ctx->vecs), 16 * P * ss))) return rc;
    if ((rc = dalloc(ctx, reinterpret_cast<unsigned char **>(&ctx->ovpart), size_t(kPartStride) * ss))) return rc;
    if ((rc = dalloc(ctx, &ctx->part, size_t(3 * kPartStride)))) return rc;
    ctx->chains = chains;
    ctx->m = m;
    ctx->arith = arith;
    ctx->Ns = Ns;
    return NQES_OK;
}

// The factors of O in the mixed form: tanh rows then coefficients, in ctx->O.
FactArgs fact_args(nqes_ctx *ctx) {
    FactArgs F{};
    F.N = ctx->sh.N;
    F.M = ctx->sh.M;
    F.K = ctx->sh.K;
    F.NW = ctx->sh.NW;
    F.Ns = int(ctx->Ns);
    F.rchunks = ctx->rchunks;
    F.MT = fact_mt(F.M);
    F.T = static_cast<const float *>(ctx->O);
    F.B = F.T + ctx->Ns * size_t(F.K) * F.K * F.MT;
    F.spins = ctx->spins;
    F.tcimg = ctx->tcimg;
    F.err = ctx->err_d;
    // the tensor-core rows pass pays off from N M = 4096 (N64 M128 K4: 1.15 -> 0.88 ms
    // per pass at 2048 x 64 samples; N32 M64 K2 stays faster on the CUDA cores)
    F.tc = ctx->tensor_cores && ctx->tcimg && rows_tc_fits(F) && (ctx->tensor_cores == 2 || F.N * F.M >= 4096);
    F.tcc = ctx->tensor_cores == 2 && cols_tc_fits(F);
    return F;
}

bool certified_dw(const nqes_ctx *ctx);
// The certified decision-warp sampler stores O as double-float pairs when the
// fused S·v reads it (NQES_OPT_FUSED_SV).
bool o_split(const nqes_ctx *ctx) { return ctx->fG > 0 && certified_dw(ctx); }

template <class S> SolveBufs<S> solve_bufs(nqes_ctx *ctx) {
    SolveBufs<S> B{};
    const size_t P = ctx->sh.P;
    B.sh = ctx->sh;
    B.Ns = int(ctx->Ns);
    B.O = static_cast<const S *>(ctx->O);
    B.E = ctx->E;
    S *vec = static_cast<S *>(ctx->vecs);
    B.o = vec + 0 * P;
    B.skk = vec + 1 * P;
    B.f = vec + 2 * P;
    B.r1 = vec + 3 * P;
    B.r2 = vec + 4 * P;
    B.r3 = vec + 5 * P;
    B.v = vec + 6 * P;
    B.vq = vec + 13 * P;  // 3 slots
    B.w = vec + 8 * P;
    B.wl = vec + 9 * P;
    B.wl2 = vec + 10 * P;
    B.x = vec + 11 * P;
    B.xl2 = vec + 12 * P;
    B.u = static_cast<S *>(ctx->u);
    B.ypart = static_cast<S *>(ctx->ypart);
    B.rchunks = ctx->rchunks;
    B.part = ctx->part;
    B.ovpart = static_cast<S *>(ctx->ovpart);
    B.qs = ctx->qs;
    B.lz = ctx->lz;
    B.sp = ctx->sp;
    B.emat = ctx->emat_d;
    B.eloc = ctx->eloc_d;
    B.err = ctx->err_d;
    B.use_cond = 0;
    B.svp = ctx->rchunks;
    B.ysv = B.ypart;
    if (std::is_same<S, double>::value && ctx->fG) {
        B.fG = ctx->fG;
        B.fNB = ctx->fNB;
        B.svp = ctx->fctas;
        B.ysv = reinterpret_cast<S *>(ctx->ysv);
        B.o_split = o_split(ctx) ? 1 : 0;
    }
    if (ctx->step_precision == NQES_PRECISION_MIXED) {
        B.O = nullptr;
        B.fact = 1;
        B.F = fact_args(ctx);
        B.v32 = ctx->v32;
        B.u32 = ctx->u32;
        B.ypart32 = ctx->ypart32;
    }
    return B;
}

bool dw_energy64(const nqes_ctx *ctx);

MixedArgs mixed_args(nqes_ctx *ctx, int chains, int m, int burn, int tk) {
    MixedArgs A{};
    A.sh = ctx->sh;
    A.chains = chains;
    A.m = m;
    A.burn = burn;
    A.tk = tk;
    A.sp = ctx->sp;
    A.ch = ctx->mch;
    A.sh32 = ctx->msh;
    A.eup = ctx->meup;
    A.edn = ctx->medn;
    A.w64 = ctx->mw;
    A.a64 = ctx->ma;
    A.b64 = ctx->mb;
    A.J = ctx->J;
    A.h = ctx->h;
    A.FT = static_cast<float *>(ctx->O);
    A.FB = A.FT + size_t(chains) * m * size_t(ctx->sh.K) * ctx->sh.K * fact_mt(ctx->sh.M);
    A.E = ctx->E;
    A.spins = ctx->spins;
    A.accepted = ctx->accepted;
    A.exact = ctx->exact;
    A.err = ctx->err_d;
    A.exact_all = ctx->mixed_exact_all ? 1 : 0;
    A.cp = ctx->dcp;
    A.cpl = ctx->dcpl;
    A.spl = ctx->dspl;
    A.spp = ctx->dsp;
    A.whp = ctx->dwh;
    A.wlp = ctx->dwl;
    A.bh = ctx->dbh;
    A.bl = ctx->dbl;
    A.bnd = ctx->dbnd;
    A.etab = ctx->etab;
    A.fdN = fast_div(unsigned(ctx->sh.N));
    A.fdM = fast_div(unsigned(ctx->sh.M));
    A.fdMP = fast_div(unsigned(std::max(ctx->dw_MP, 1)));
    A.fdMT = fast_div(unsigned(fact_mt(ctx->sh.M)));
    A.G = ctx->dw_G;
    A.U = ctx->dw_U;
    A.MP = ctx->dw_MP;
    A.stage_fault = ctx->stage_fault;
    A.o_split = o_split(ctx) ? 1 : 0;
    A.out64 = ctx->step_precision == NQES_PRECISION_CERTIFIED ? 1 : 0;
    A.e64 = !A.out64 && dw_energy64(ctx) ? ctx->mixed_e64 : 0;
    if (A.e64) {  // the FP64 tables for the local energies; O stays as FP32 factors
        const size_t nw = size_t(ctx->sh.K) * ctx->sh.N * ctx->sh.M, na = size_t(ctx->sh.K) * ctx->sh.N;
        const double *t = static_cast<const double *>(ctx->tab);
        A.c64 = t;
        A.s64 = t + nw;
        A.eup64 = t + 2 * nw;
        A.edn64 = t + 2 * nw + na;
    }
    if (A.out64) {
        // dense FP64 O and the FP64 tables of the step (ch, sh, eup, edn)
        const size_t nw = size_t(ctx->sh.K) * ctx->sh.N * ctx->sh.M, na = size_t(ctx->sh.K) * ctx->sh.N;
        const double *t = static_cast<const double *>(ctx->tab);
        A.O64 = static_cast<double *>(ctx->O);
        A.FT = A.FB = nullptr;
        A.c64 = t;
        A.s64 = t + nw;
        A.eup64 = t + 2 * nw;
        A.edn64 = t + 2 * nw + na;
    }
    return A;
}

// The decision-warp sampler (certified FP32 decisions) runs for MIXED and, with
// FP64 outputs, for CERTIFIED with real arithmetic on the shapes it covers; a
// CERTIFIED step beyond those runs the FP64 sampler.
bool certified_dw(const nqes_ctx *ctx) {
    return ctx->step_precision == NQES_PRECISION_CERTIFIED && ctx->dw_U && ctx->arith == NQES_ARITH_REAL;
}
bool uses_mixed_sampler(const nqes_ctx *ctx) {
    return ctx->step_precision == NQES_PRECISION_MIXED || certified_dw(ctx);
}
// The decision-warp sampler forms its local energies in FP64 (the certified
// form; the mixed form unless NQES_OPT_MIXED_ENERGY64 is 0): it then needs the
// FP64 tables and room for FP64 tanh rows.
bool dw_energy64(const nqes_ctx *ctx) {
    return certified_dw(ctx) || (ctx->step_precision == NQES_PRECISION_MIXED && ctx->dw_U && ctx->mixed_e64 != 0);
}

cudaError_t launch_tables_mixed_ctx(nqes_ctx *ctx) {
    return launch_tables_mixed(ctx->sh, ctx->a, ctx->b, ctx->w, ctx->mch, ctx->msh, ctx->meup, ctx->medn, ctx->mw,
                               ctx->ma, ctx->mb, ctx->st);
}

// Launch plan of the decision-warp sampler: warps per chain (the warps past
// the first rebuild rows and form samples) and whether the step's tables are
// bulk-copied into shared memory. The first plan, in the order (4 warps,
// staged), (4, global), (2, staged), ..., under which every chain gets a
// resident CTA; else 1 warp reading global memory.
void dw_plan(nqes_ctx *ctx, int chains, int *warps, int *stage) {
    if (ctx->dw_force_warps) {
        *warps = ctx->dw_force_warps;
        *stage = ctx->dw_force_stage;
        return;
    }
    if (ctx->stage_fault) {  // test hook: a staged plan, so that the staging wait exists
        *warps = 1;
        *stage = 1;
        return;
    }
    if (ctx->plan_chains) chains = ctx->plan_chains;
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    // the certified form's samples (FP64 tanh and flip ratios, the O row) go to
    // the helper warps beside the sweep: seven helpers keep them off its path
    // (128 chains at N32 M64 K2: 12.9 against 14.8 ms with three); the mixed
    // form's lighter samples gain nothing from more than four warps
    const int wmax = certified_dw(ctx) ? 8 : 4;
    for (int w = wmax; w >= 1; w >>= 1)
        for (int st = 1; st >= 0; st--) {
            const size_t smem = dw_smem_bytes(ctx->sh, ctx->dw_MP, st == 1, dw_energy64(ctx));
            if (smem > 227 * 1024) continue;
            int per_sm = 0;
            if (dw_occupancy(ctx->sh, 32 * w, smem, &per_sm) == cudaSuccess && per_sm * sms >= chains) {
                *warps = w;
                *stage = st;
                return;
            }
        }
    *warps = 1;
    *stage = 0;
}

// The mixed sampler's tables, its shared-memory attribute and its launch,
// in the decision-warp form when it applies, else the block form.
cudaError_t launch_mixed_tables(nqes_ctx *ctx) {
    cudaError_t e = launch_tables_mixed_ctx(ctx);
    if (e == cudaSuccess && ctx->dw_U)
        e = launch_tables_dw(ctx->sh, ctx->dw_MP, ctx->b, ctx->w, ctx->dcp, ctx->dsp, ctx->dwh, ctx->dwl, ctx->dbh,
                             ctx->dbl, ctx->dbnd, ctx->dcpl, ctx->dspl, ctx->st);
    return e;
}
size_t mixed_sampler_smem(nqes_ctx *ctx) {
    return ctx->dw_U ? dw_smem_bytes(ctx->sh, ctx->dw_MP, false, dw_energy64(ctx)) : mixed_smem_bytes(ctx->sh);
}
// The mixed sampler's and the factored S·v's shared-memory limits.
cudaError_t prepare_mixed_sampler(nqes_ctx *ctx) {
    FactArgs F{};
    F.N = ctx->sh.N;
    F.M = ctx->sh.M;
    F.K = ctx->sh.K;
    cudaError_t e = prepare_frows(F);
    if (e != cudaSuccess) return e;
    return ctx->dw_U ? prepare_sample_dw(ctx->sh, ctx->dw_MP) : prepare_sample_mixed(ctx->sh);
}
cudaError_t launch_mixed_sampler(nqes_ctx *ctx, int chains, int m, int burn, int tk) {
    MixedArgs A = mixed_args(ctx, chains, m, burn, tk);
    if (!ctx->dw_U) return launch_sample_mixed(A, ctx->st);
    int warps = 1;
    dw_plan(ctx, chains, &warps, &A.stage);
    return launch_sample_dw(A, warps, ctx->st);
}

template <class S> Tables<S> tables(nqes_ctx *ctx) {
    const size_t nw = size_t(ctx->sh.K) * ctx->sh.N * ctx->sh.M, na = size_t(ctx->sh.K) * ctx->sh.N;
    S *t = static_cast<S *>(ctx->tab);
    return Tables<S>{t, t + nw, t + 2 * nw, t + 2 * nw + na};
}

template <class S> SampleArgs<S> sample_args(nqes_ctx *ctx, int chains, int m, int burn, int tk) {
    SampleArgs<S> A{};
    A.sh = ctx->sh;
    A.chains = chains;
    A.m = m;
    A.burn = burn;
    A.tk = tk;
    A.sp = ctx->sp;
    A.tab = tables<S>(ctx);
    A.a = ctx->a;
    A.b = ctx->b;
    A.w = ctx->w;
    A.J = ctx->J;
    A.h = ctx->h;
    A.ham = ctx->ham;
    A.delta = ctx->ham_delta;
    A.O = static_cast<S *>(ctx->O);
    A.E = ctx->E;
    A.spins = ctx->spins;
    A.accepted = ctx->accepted;
    A.err = ctx->err_d;
    if (std::is_same<S, double>::value && ctx->reject_filter) {
        A.c32 = ctx->mch;
        A.s32 = ctx->msh;
        A.eu32 = ctx->meup;
        A.ed32 = ctx->medn;
    }
    return A;
}

// The sampler's per-step tables; with the rejection filter (real arithmetic)
// also their FP32 roundings.
template <class S> cudaError_t launch_tables_ctx(nqes_ctx *ctx) {
    Tables<S> t = tables<S>(ctx);
    cudaError_t e = launch_tables<S>(ctx->sh, ctx->a, ctx->w, const_cast<S *>(t.ch), const_cast<S *>(t.sh),
                                     const_cast<S *>(t.eup), const_cast<S *>(t.edn), ctx->st);
    if (e == cudaSuccess && std::is_same<S, double>::value && ctx->reject_filter) e = launch_tables_mixed_ctx(ctx);
    return e;
}

// Threads per RBM column block (TK): at most eight hidden units per thread,
// K*TK <= 256 unit threads; wide blocks when there are few chains to spread
// over the SMs (latency), narrow ones when chains fill the GPU (throughput).
int choose_tk(nqes_ctx *ctx, int chains) {
    const int M = ctx->sh.M, K = ctx->sh.K;
    const int tmin = std::max(32, ((M + 7) / 8 + 31) / 32 * 32);
    const int tmax = std::max(32, 256 / K / 32 * 32);
    int tk;
    if (ctx->tk_opt) {
        tk = ctx->tk_opt;
    } else if (ctx->tk_tuned) {
        tk = ctx->tk_tuned;
    } else {
        int dev_sms = 152;
        cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, ctx->device);
        if (ctx->plan_chains) chains = ctx->plan_chains;
        tk = chains <= dev_sms ? std::min(128, (M + 31) / 32 * 32) : tmin;
    }
    return std::min(std::max(tk, tmin), tmax);
}

// Captures the sampling segment of one SR step into *out: the error word
// cleared, the tables, the sampler, the moments, and the MINRES-QLP init with
// the first Lanczos step. Sets the sampler's shared-memory attribute first
// (that call is not allowed during a capture).
template <class S> int capture_sampling(nqes_ctx *ctx, int chains, int m, int burn, int tk, cudaGraph_t *out) {
    SampleArgs<S> A = sample_args<S>(ctx, chains, m, burn, tk);
    SolveBufs<S> B = solve_bufs<S>(ctx);
    const int threads = sample_threads(ctx->sh.K, tk);
    {
        const bool mixed = uses_mixed_sampler(ctx);
        const size_t smem = mixed ? mixed_sampler_smem(ctx) : sample_smem_bytes(ctx->sh, threads, sizeof(S) == sizeof(cplx));
        if (smem > 227 * 1024) {
            ctx->err = "shape needs " + std::to_string(smem) + " bytes of shared memory per chain";
            return NQES_ERR_INVALID;
        }
        if (mixed)
            NQES_CUDA(prepare_mixed_sampler(ctx));
        else
            NQES_CUDA(prepare_sample<S>(ctx->sh));
    }
    NQES_CUDA(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    cudaMemsetAsync(ctx->err_d, 0, sizeof(int), ctx->st);
    cudaError_t le;
    if (uses_mixed_sampler(ctx)) {
        le = launch_mixed_tables(ctx);
        if (le == cudaSuccess && dw_energy64(ctx)) le = launch_tables_ctx<S>(ctx);  // the FP64 energies' tables
        if (le == cudaSuccess) le = launch_mixed_sampler(ctx, chains, m, burn, tk);
    } else {
        le = launch_tables_ctx<S>(ctx);
        if (le == cudaSuccess) le = launch_sample<S>(A, threads, ctx->st);
    }
    if (le == cudaSuccess) le = launch_moments<S>(B, ctx->st);
    if (le == cudaSuccess) le = launch_minres_init<S>(B, ctx->st);
    const cudaError_t ce = cudaStreamEndCapture(ctx->st, out);
    if (le != cudaSuccess || ce != cudaSuccess) {
        ctx->err = std::string("capture of the sampling segment: ") + cudaGetErrorString(le != cudaSuccess ? le : ce);
        if (ce == cudaSuccess && *out) cudaGraphDestroy(*out);
        *out = nullptr;
        return NQES_ERR_CUDA;
    }
    return NQES_OK;
}

// Captures the update w -= lr x into *out.
template <class S> int capture_update(nqes_ctx *ctx, cudaGraph_t *out) {
    SolveBufs<S> B = solve_bufs<S>(ctx);
    NQES_CUDA(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    const cudaError_t le = launch_update<S>(ctx->sh, ctx->sp, B.x, ctx->a, ctx->b, ctx->w, ctx->st);
    const cudaError_t ce = cudaStreamEndCapture(ctx->st, out);
    if (le != cudaSuccess || ce != cudaSuccess) {
        ctx->err = std::string("capture of the update: ") + cudaGetErrorString(le != cudaSuccess ? le : ce);
        if (ce == cudaSuccess && *out) cudaGraphDestroy(*out);
        *out = nullptr;
        return NQES_ERR_CUDA;
    }
    return NQES_OK;
}

// Appends one SR step of ctx to graph g as three nodes with no dependency on
// anything else in g: the sampling segment (tables, sampler, moments, MINRES
// init), a conditional while node running the MINRES-QLP body, the update.
template <class S> int add_step_nodes(nqes_ctx *ctx, cudaGraph_t g, int chains, int m, int burn, int tk) {
    SolveBufs<S> B = solve_bufs<S>(ctx);
    cudaGraph_t gA = nullptr, gC = nullptr;
    int rc = capture_sampling<S>(ctx, chains, m, burn, tk, &gA);
    if (rc) return rc;
    cudaGraphConditionalHandle cond;
    // Default value 1 on every launch: the body runs at least once, and its
    // scalar kernel writes 0 as soon as the solve has finished (or was
    // never needed), so the loop always ends.
    NQES_CUDA(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNode_t nA, nW, nC;
    NQES_CUDA(cudaGraphAddChildGraphNode(&nA, g, nullptr, 0, gA));
    cudaGraphDestroy(gA);
    cudaGraphNodeParams cp{};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = cond;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    NQES_CUDA(cudaGraphAddNode(&nW, g, &nA, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    B.cond = cond;
    B.use_cond = 1;
    // Loop body: the Lanczos step j + 1 on st beside the QLP step j (whose
    // scalar kernel sets the loop condition) on st_qlp; the first Lanczos step
    // ran before the loop.
    NQES_CUDA(cudaStreamBeginCaptureToGraph(ctx->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    cudaError_t le = cudaEventRecord(ctx->ev_fork, ctx->st);
    if (le == cudaSuccess) le = cudaStreamWaitEvent(ctx->st_qlp, ctx->ev_fork, 0);
    if (le == cudaSuccess) le = launch_qlp_step<S>(B, ctx->st_qlp);
    if (le == cudaSuccess) le = launch_lanczos_step<S>(B, ctx->st);
    if (le == cudaSuccess) le = cudaEventRecord(ctx->ev_join, ctx->st_qlp);
    if (le == cudaSuccess) le = cudaStreamWaitEvent(ctx->st, ctx->ev_join, 0);
    cudaError_t ce = cudaStreamEndCapture(ctx->st, &body);
    if (le != cudaSuccess || ce != cudaSuccess) {
        ctx->err = std::string("capture of the MINRES-QLP body: ") + cudaGetErrorString(le != cudaSuccess ? le : ce);
        return NQES_ERR_CUDA;
    }
    if ((rc = capture_update<S>(ctx, &gC))) return rc;
    NQES_CUDA(cudaGraphAddChildGraphNode(&nC, g, &nW, 1, gC));
    cudaGraphDestroy(gC);
    return NQES_OK;
}

// ---- pieces of the batch graph (one shared MINRES-QLP loop) ----

// The member's sampling segment as a node of g with no dependencies.
template <class S>
int add_member_sampling(nqes_ctx *ctx, cudaGraph_t g, int chains, int m, int burn, int tk, cudaGraphNode_t *node) {
    cudaGraph_t gA = nullptr;
    const int rc = capture_sampling<S>(ctx, chains, m, burn, tk, &gA);
    if (rc) return rc;
    const cudaError_t e = cudaGraphAddChildGraphNode(node, g, nullptr, 0, gA);
    cudaGraphDestroy(gA);
    if (e != cudaSuccess) {
        ctx->err = std::string("cudaGraphAddChildGraphNode: ") + cudaGetErrorString(e);
        return NQES_ERR_CUDA;
    }
    return NQES_OK;
}

// The member's update as a node of g after `after`.
template <class S> int add_member_update(nqes_ctx *ctx, cudaGraph_t g, cudaGraphNode_t after) {
    cudaGraph_t gC = nullptr;
    const int rc = capture_update<S>(ctx, &gC);
    if (rc) return rc;
    cudaGraphNode_t nC;
    const cudaError_t e = cudaGraphAddChildGraphNode(&nC, g, &after, 1, gC);
    cudaGraphDestroy(gC);
    if (e != cudaSuccess) {
        ctx->err = std::string("cudaGraphAddChildGraphNode: ") + cudaGetErrorString(e);
        return NQES_ERR_CUDA;
    }
    return NQES_OK;
}

// Address of the member's QlpState::running in device memory.
const int *running_flag(const nqes_ctx *ctx) {
    return reinterpret_cast<const int *>(reinterpret_cast<const char *>(ctx->qs) + offsetof(QlpState, running));
}

template <class S> int build_graph(nqes_ctx *ctx, int chains, int m, int burn, int tk) {
    if (ctx->exec) {
        cudaGraphExecDestroy(ctx->exec);
        ctx->exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    NQES_CUDA(cudaGraphCreate(&g, 0));
    int rc = add_step_nodes<S>(ctx, g, chains, m, burn, tk);
    if (rc == NQES_OK && cudaGraphInstantiate(&ctx->exec, g, 0) != cudaSuccess) {
        ctx->err = "cudaGraphInstantiate failed";
        rc = NQES_ERR_CUDA;
    }
    cudaGraphDestroy(g);
    if (rc) return rc;
    ctx->g_chains = chains;
    ctx->g_m = m;
    ctx->g_burn = burn;
    ctx->g_arith = ctx->arith;
    ctx->g_tk = tk;
    ctx->g_prec = ctx->step_precision;
    return NQES_OK;
}

bool host_weights_real(const double *a, const double *b, const double *w, const Shape &sh) {
    auto check = [](const double *p, size_t n) {
        for (size_t t = 0; t < n; t++)
            if (p[2 * t + 1] != 0.0) return false;
        return true;
    };
    return check(a, size_t(sh.K) * sh.N) && check(b, size_t(sh.K) * sh.M) && check(w, size_t(sh.K) * sh.N * sh.M);
}

int resolve_arith(nqes_ctx *ctx) {
    if (ctx->arith_opt == NQES_ARITH_COMPLEX) return NQES_ARITH_COMPLEX;
    if (ctx->arith_opt == NQES_ARITH_REAL) return NQES_ARITH_REAL;
    return ctx->weights_real ? NQES_ARITH_REAL : NQES_ARITH_COMPLEX;
}

// Copy an S-typed device array to interleaved complex host memory.
int copy_out_c(nqes_ctx *ctx, const void *src, size_t n, double *dst) {
    if (ctx->arith == NQES_ARITH_COMPLEX) {
        NQES_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(cplx), cudaMemcpyDeviceToHost, ctx->st));
        NQES_CUDA(cudaStreamSynchronize(ctx->st));
    } else {
        std::vector<double> tmp(n);
        NQES_CUDA(cudaMemcpyAsync(tmp.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
        NQES_CUDA(cudaStreamSynchronize(ctx->st));
        for (size_t t = 0; t < n; t++) {
            dst[2 * t] = tmp[t];
            dst[2 * t + 1] = 0.0;
        }
    }
    return NQES_OK;
}

// ---- one SR step in pieces (shared by nqes_sr_step and the batch) ----

template <class S> int tune_sampler(nqes_ctx *ctx, int chains, int m, int burn);

// Validates the arguments, sizes the step buffers, fills the step scalars and,
// with NQES_OPT_AUTOTUNE, picks the sampler's launch shape by timing.
int step_prepare(nqes_ctx *ctx, uint64_t seed, int chains, int m, int burn, double lr, double reglam, double rtol,
                 uint64_t maxit, int *arith_out) {
    if (chains < 1 || m < 1 || burn < 0 || !std::isfinite(lr) || !std::isfinite(reglam) || !(rtol >= 0)) {
        ctx->err = "invalid SR step arguments (chains >= 1, m >= 1, burn_in >= 0, finite lr/reglam, rtol >= 0)";
        return NQES_ERR_INVALID;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    const int arith = resolve_arith(ctx);
    if (ctx->precision == NQES_PRECISION_MIXED && arith != NQES_ARITH_REAL) {
        ctx->err = "mixed precision needs real weights (NQES_ARITH_REAL)";
        return NQES_ERR_INVALID;
    }
    if (ctx->ham != NQES_HAM_ISING_LIKE && ctx->precision != NQES_PRECISION_FP64) {
        ctx->err = "the Heisenberg-like local energy runs in the FP64 form (NQES_PRECISION_FP64)";
        return NQES_ERR_INVALID;
    }
    int rc = ensure_step_buffers(ctx, chains, m, arith);
    if (rc) return rc;
    StepParams &p = *ctx->sp_host;
    p.seed = seed;
    p.lr = lr;
    p.reglam = reglam;
    p.rtol = rtol;
    p.maxit = std::min<uint64_t>(maxit, ctx->minres_cap);
    *arith_out = arith;
    if (ctx->autotune) {
        const long long key[5] = {chains, m, burn, ctx->step_precision, arith};
        if (!std::equal(key, key + 5, ctx->tune_key)) {
            rc = arith == NQES_ARITH_COMPLEX ? tune_sampler<cplx>(ctx, chains, m, burn)
                                             : tune_sampler<double>(ctx, chains, m, burn);
            if (rc) return rc;
            std::copy(key, key + 5, ctx->tune_key);
        }
    }
    return NQES_OK;
}

// Queues the copies of the step's results to pinned host memory on stream st.
int step_readback(nqes_ctx *ctx, cudaStream_t st) {
    NQES_CUDA(cudaMemcpyAsync(ctx->emat_host, ctx->emat_d, sizeof(cplx) * ctx->sh.K * ctx->sh.K,
                              cudaMemcpyDeviceToHost, st));
    NQES_CUDA(cudaMemcpyAsync(ctx->emat_host + 16, ctx->eloc_d, sizeof(cplx), cudaMemcpyDeviceToHost, st));
    NQES_CUDA(cudaMemcpyAsync(ctx->qs_host, ctx->qs, sizeof(QlpState), cudaMemcpyDeviceToHost, st));
    NQES_CUDA(cudaMemcpyAsync(ctx->err_host, ctx->err_d, sizeof(int), cudaMemcpyDeviceToHost, st));
    return NQES_OK;
}

// After the step's stream has drained: e_mat, the step report, error bits.
int step_finish(nqes_ctx *ctx, int chains, int m, int burn, int arith, uint64_t maxit, float ms, double *e_mat,
                nqes_step_info *info) {
    ctx->have_step = true;
    ctx->last_burn = burn;
    if (e_mat) std::memcpy(e_mat, ctx->emat_host, sizeof(cplx) * ctx->sh.K * ctx->sh.K);
    const QlpState &q = *ctx->qs_host;
    if (info) {
        std::memset(info, 0, sizeof(*info));
        info->minres_flag = q.flag;
        info->arith = arith;
        info->minres_iters = q.iters;
        info->qlp_iters = q.qlp_iters;
        info->relres = q.relres;
        info->anorm = q.anorm;
        info->acond = q.acond;
        info->xnorm = q.xnorm;
        info->proposals = uint64_t(chains) * (burn + m) * ctx->sh.K * ctx->sh.N;
        info->eloc_re = ctx->emat_host[16].re;
        info->eloc_im = ctx->emat_host[16].im;
        info->ms_total = ms;
        std::vector<unsigned long long> acc(chains);
        NQES_CUDA(cudaMemcpy(acc.data(), ctx->accepted, sizeof(unsigned long long) * chains, cudaMemcpyDeviceToHost));
        for (auto x : acc) info->accepted += x;
        if (q.flag == 8 && q.iters >= ctx->minres_cap && maxit > ctx->minres_cap) info->warnings |= 1;
        // tables, sampler, 3 moment kernels, 3 MINRES-QLP init kernels, the
        // first Lanczos step (5), update, and 7 kernels per execution of the
        // loop body (Lanczos step 5, QLP step 2)
        info->kernel_launches = 14 + 7 * q.bodies;
        info->precision = ctx->step_precision;
        if (uses_mixed_sampler(ctx)) {
            std::vector<unsigned long long> ex(chains);
            NQES_CUDA(cudaMemcpy(ex.data(), ctx->exact, sizeof(unsigned long long) * chains, cudaMemcpyDeviceToHost));
            for (auto x : ex) info->exact_decisions += x;
        }
    }
    const int e = *ctx->err_host;
    if (e & kErrLaunch) {  // a kernel returned at entry: the step's results are not meaningful
        ctx->err = "a kernel was launched with less dynamic shared memory than its layout needs (launch check)";
        return NQES_ERR_CUDA;
    }
    if (e & kErrTimeout) {  // what the step computed after a wait ran out is not meaningful
        ctx->err = "a bounded device-side wait ran out (bulk staging into shared memory)";
        return NQES_ERR_TIMEOUT;
    }
    if (e & (kErrNonFinite | kErrMinresNonFinite)) {
        ctx->err = "non-finite value during the SR step (error bits " + std::to_string(e) + ")";
        return NQES_ERR_NONFINITE;
    }
    if (e & kErrSingular) {
        ctx->err = "a sample was taken at a singular Phi";
        return NQES_ERR_NONFINITE;
    }
    return NQES_OK;
}

// Autotuner: times the sampler alone (tables built, a shortened chain of
// min(m, 8) samples after min(burn, 2) sweeps) for every admissible launch
// shape and keeps the fastest: threads per column block for the FP64 and
// block-form mixed samplers, (warps per chain, table staging) for the
// decision-warp sampler.
template <class S> int tune_sampler(nqes_ctx *ctx, int chains, int m, int burn) {
    const int mt = std::min(m, 8), bt = std::min(burn, 2);
    const bool mixed = uses_mixed_sampler(ctx);
    NQES_CUDA(cudaMemcpyAsync(ctx->sp, ctx->sp_host, sizeof(StepParams), cudaMemcpyHostToDevice, ctx->st));
    if (mixed) NQES_CUDA(launch_mixed_tables(ctx));
    if (!mixed || dw_energy64(ctx)) NQES_CUDA(launch_tables_ctx<S>(ctx));
    auto time_one = [&](auto &&launch, float *ms) -> cudaError_t {
        cudaError_t e = launch();  // warm-up
        if (e != cudaSuccess) return e;
        cudaEventRecord(ctx->ev0, ctx->st);
        e = launch();
        cudaEventRecord(ctx->ev1, ctx->st);
        if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1);
        return e;
    };
    float best = 1e30f;
    if (mixed && ctx->dw_U) {
        NQES_CUDA(prepare_mixed_sampler(ctx));
        int bw = 0, bs = 0;
        for (int w = 1; w <= (certified_dw(ctx) ? 8 : 4); w <<= 1)
            for (int st = 0; st <= 1; st++) {
                if (dw_smem_bytes(ctx->sh, ctx->dw_MP, st == 1, dw_energy64(ctx)) > 227 * 1024) continue;
                ctx->dw_force_warps = w;
                ctx->dw_force_stage = st;
                float ms = 0;
                NQES_CUDA(time_one([&] { return launch_mixed_sampler(ctx, chains, mt, bt, 0); }, &ms));
                if (ms < best) {
                    best = ms;
                    bw = w;
                    bs = st;
                }
            }
        ctx->dw_force_warps = bw;
        ctx->dw_force_stage = bs;
        return NQES_OK;
    }
    const int M = ctx->sh.M, K = ctx->sh.K;
    const int tmin = std::max(32, ((M + 7) / 8 + 31) / 32 * 32), tmax = std::max(32, 256 / K / 32 * 32);
    if (mixed)
        NQES_CUDA(prepare_mixed_sampler(ctx));
    else
        NQES_CUDA(prepare_sample<S>(ctx->sh));
    int bt_k = tmin;
    for (int tk = tmin; tk <= tmax; tk += 32) {
        float ms = 0;
        if (mixed) {
            NQES_CUDA(time_one([&] { return launch_sample_mixed(mixed_args(ctx, chains, mt, bt, tk), ctx->st); }, &ms));
        } else {
            const SampleArgs<S> A = sample_args<S>(ctx, chains, mt, bt, tk);
            NQES_CUDA(time_one([&] { return launch_sample<S>(A, sample_threads(K, tk), ctx->st); }, &ms));
        }
        if (ms < best) {
            best = ms;
            bt_k = tk;
        }
    }
    ctx->tk_tuned = bt_k;
    return NQES_OK;
}

template <class S> int sr_step_t(nqes_ctx *ctx, int chains, int m, int burn) {
    const int tk = choose_tk(ctx, chains);
    if (!ctx->exec || ctx->g_chains != chains || ctx->g_m != m || ctx->g_burn != burn || ctx->g_arith != ctx->arith ||
        ctx->g_tk != tk || ctx->g_prec != ctx->step_precision) {
        int rc = build_graph<S>(ctx, chains, m, burn, tk);
        if (rc) return rc;
    }
    ctx->last_tk = tk;
    NQES_CUDA(cudaMemcpyAsync(ctx->sp, ctx->sp_host, sizeof(StepParams), cudaMemcpyHostToDevice, ctx->st));
    NQES_CUDA(cudaEventRecord(ctx->ev0, ctx->st));
    NQES_CUDA(cudaGraphLaunch(ctx->exec, ctx->st));
    NQES_CUDA(cudaEventRecord(ctx->ev1, ctx->st));
    return NQES_OK;
}

}  // namespace

extern "C" {

const char *nqes_last_error(const nqes_ctx *ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int nqes_create(int N, int M, int K, const double *J, double h, int device, nqes_ctx **out) {
    if (!out) {
        g_create_error = "out is NULL";
        return NQES_ERR_INVALID;
    }
    *out = nullptr;
    if (K < 1 || K > 4 || N < 1 || N > 128 || M < 1 || M > 512 || !J) {
        g_create_error = "shape out of range (1<=K<=4, 1<=N<=128, 1<=M<=512) or J is NULL";
        return NQES_ERR_INVALID;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || device < 0 || device >= ndev) {
        g_create_error = "no CUDA device " + std::to_string(device);
        return NQES_ERR_CUDA;
    }
    nqes_ctx *ctx = new nqes_ctx();
    ctx->device = device;
    ctx->h = h;
    ctx->sh = Shape{N, M, K, N + M + N * M, K * (N + M + N * M), (N + 63) / 64};
    auto fail = [&](int rc) {
        g_create_error = ctx->err;
        nqes_destroy(ctx);
        return rc;
    };
    if (cudaSetDevice(device) != cudaSuccess) {
        ctx->err = "cudaSetDevice failed";
        return fail(NQES_ERR_CUDA);
    }
    if (cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking) != cudaSuccess) {
        ctx->err = "cudaStreamCreate failed";
        return fail(NQES_ERR_CUDA);
    }
    if (cudaStreamCreateWithFlags(&ctx->st_qlp, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess) {
        ctx->err = "cudaStreamCreate / cudaEventCreate failed";
        return fail(NQES_ERR_CUDA);
    }
    cudaEventCreate(&ctx->ev0);
    cudaEventCreate(&ctx->ev1);
    const size_t nw = size_t(K) * N * M, na = size_t(K) * N;
    int rc;
    if ((rc = dalloc(ctx, &ctx->a, na)) || (rc = dalloc(ctx, &ctx->b, size_t(K) * M)) ||
        (rc = dalloc(ctx, &ctx->w, nw)) || (rc = dalloc(ctx, &ctx->J, size_t(N) * N)) ||
        (rc = dalloc(ctx, reinterpret_cast<cplx **>(&ctx->tab), 2 * nw + 2 * na)) ||
        (rc = dalloc(ctx, &ctx->sp, 1)) || (rc = dalloc(ctx, &ctx->qs, 1)) || (rc = dalloc(ctx, &ctx->lz, 1)) ||
        (rc = dalloc(ctx, &ctx->err_d, 1)) ||
        (rc = dalloc(ctx, &ctx->emat_d, 16)) || (rc = dalloc(ctx, &ctx->eloc_d, 1)) ||
        (rc = dalloc(ctx, &ctx->mch, nw)) || (rc = dalloc(ctx, &ctx->msh, nw)) || (rc = dalloc(ctx, &ctx->meup, na)) ||
        (rc = dalloc(ctx, &ctx->medn, na)) || (rc = dalloc(ctx, &ctx->mw, nw)) || (rc = dalloc(ctx, &ctx->ma, na)) ||
        (rc = dalloc(ctx, &ctx->mb, size_t(K) * M)))
        return fail(rc);
    ctx->dw_U = dw_units(ctx->sh, &ctx->dw_G);
    if (ctx->dw_U) {
        ctx->dw_MP = ctx->dw_G * ctx->dw_U;
        const size_t np = size_t(K) * N * ctx->dw_MP, nb = size_t(K) * ctx->dw_MP;
        if ((rc = dalloc(ctx, &ctx->dcp, np)) || (rc = dalloc(ctx, &ctx->dsp, np)) || (rc = dalloc(ctx, &ctx->dwh, np)) ||
            (rc = dalloc(ctx, &ctx->dcpl, np)) || (rc = dalloc(ctx, &ctx->dspl, np)) ||
            (rc = dalloc(ctx, &ctx->dwl, np)) || (rc = dalloc(ctx, &ctx->dbh, nb)) || (rc = dalloc(ctx, &ctx->dbl, nb)) ||
            (rc = dalloc(ctx, &ctx->dbnd, 4 * size_t(K) * N + 4 * size_t(K))) ||
            (rc = dalloc(ctx, &ctx->etab, size_t(kExpTabN))))
            return fail(rc);
        if (launch_exp_table(ctx->etab, ctx->st) != cudaSuccess || cudaStreamSynchronize(ctx->st) != cudaSuccess) {
            ctx->err = "exp table kernel failed";
            return fail(NQES_ERR_CUDA);
        }
    }
    if (cudaMallocHost(&ctx->sp_host, sizeof(StepParams)) != cudaSuccess ||
        cudaMallocHost(&ctx->qs_host, sizeof(QlpState)) != cudaSuccess ||
        cudaMallocHost(&ctx->err_host, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&ctx->emat_host, 17 * sizeof(cplx)) != cudaSuccess) {
        ctx->err = "cudaMallocHost failed";
        return fail(NQES_ERR_OOM);
    }
    if (cudaMemcpy(ctx->J, J, sizeof(double) * N * N, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(ctx->a, 0, sizeof(cplx) * na) != cudaSuccess ||
        cudaMemset(ctx->b, 0, sizeof(cplx) * K * M) != cudaSuccess ||
        cudaMemset(ctx->w, 0, sizeof(cplx) * nw) != cudaSuccess) {
        ctx->err = "initial copies failed";
        return fail(NQES_ERR_CUDA);
    }
    *out = ctx;
    return NQES_OK;
}

int nqes_destroy(nqes_ctx *ctx) {
    if (!ctx) return NQES_OK;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    free_step_buffers(ctx);
    dfree(ctx->a);
    dfree(ctx->b);
    dfree(ctx->w);
    dfree(ctx->J);
    dfree(ctx->tab);
    dfree(ctx->mch);
    dfree(ctx->msh);
    dfree(ctx->meup);
    dfree(ctx->medn);
    dfree(ctx->mw);
    dfree(ctx->ma);
    dfree(ctx->mb);
    dfree(ctx->dcp);
    dfree(ctx->dcpl);
    dfree(ctx->dspl);
    dfree(ctx->dsp);
    dfree(ctx->dwh);
    dfree(ctx->dwl);
    dfree(ctx->dbh);
    dfree(ctx->dbl);
    dfree(ctx->dbnd);
    dfree(ctx->etab);
    dfree(ctx->sp);
    dfree(ctx->qs);
    dfree(ctx->lz);
    dfree(ctx->err_d);
    dfree(ctx->emat_d);
    dfree(ctx->eloc_d);
    if (ctx->sp_host) cudaFreeHost(ctx->sp_host);
    if (ctx->qs_host) cudaFreeHost(ctx->qs_host);
    if (ctx->err_host) cudaFreeHost(ctx->err_host);
    if (ctx->emat_host) cudaFreeHost(ctx->emat_host);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->st_qlp) cudaStreamDestroy(ctx->st_qlp);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
    return NQES_OK;
}

int nqes_set_hamiltonian(nqes_ctx *ctx, int form, double delta) {
    if (!ctx) return NQES_ERR_INVALID;
    if ((form != NQES_HAM_ISING_LIKE && form != NQES_HAM_HEISENBERG_LIKE) || !std::isfinite(delta)) {
        ctx->err = "hamiltonian form must be NQES_HAM_ISING_LIKE or NQES_HAM_HEISENBERG_LIKE, delta finite";
        return NQES_ERR_INVALID;
    }
    ctx->ham = form;
    ctx->ham_delta = delta;
    if (ctx->exec) {  // the captured step bakes the sampler's arguments in
        cudaGraphExecDestroy(ctx->exec);
        ctx->exec = nullptr;
    }
    return NQES_OK;
}

int nqes_set_option(nqes_ctx *ctx, int option, int64_t value) {
    if (!ctx) return NQES_ERR_INVALID;
    switch (option) {
    case NQES_OPT_ARITH:
        if (value < 0 || value > 2) {
            ctx->err = "arith must be AUTO, COMPLEX or REAL";
            return NQES_ERR_INVALID;
        }
        if (value == NQES_ARITH_REAL && !ctx->weights_real) {
            ctx->err = "weights have non-zero imaginary parts; real arithmetic refused";
            return NQES_ERR_INVALID;
        }
        ctx->arith_opt = int(value);
        return NQES_OK;
    case NQES_OPT_THREADS_PER_BLOCK:
        if (value != 0 && value != 32 && value != 64 && value != 96 && value != 128) {
            ctx->err = "threads per column block must be 0 (auto), 32, 64, 96 or 128";
            return NQES_ERR_INVALID;
        }
        ctx->tk_opt = int(value);
        return NQES_OK;
    case NQES_OPT_MINRES_CAP:
        if (value < 1) {
            ctx->err = "MINRES cap must be positive";
            return NQES_ERR_INVALID;
        }
        ctx->minres_cap = uint64_t(value);
        return NQES_OK;
    case NQES_OPT_PRECISION:
        if (value != NQES_PRECISION_FP64 && value != NQES_PRECISION_MIXED && value != NQES_PRECISION_CERTIFIED) {
            ctx->err = "precision must be NQES_PRECISION_FP64, NQES_PRECISION_MIXED or NQES_PRECISION_CERTIFIED";
            return NQES_ERR_INVALID;
        }
        ctx->precision = int(value);
        return NQES_OK;
    case NQES_OPT_AUTOTUNE:
        if (value != 0 && value != 1) {
            ctx->err = "option value must be 0 or 1";
            return NQES_ERR_INVALID;
        }
        ctx->autotune = value == 1;
        std::fill(ctx->tune_key, ctx->tune_key + 5, -1LL);
        ctx->tk_tuned = ctx->dw_force_warps = ctx->dw_force_stage = 0;
        if (ctx->exec) {
            cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
        }
        return NQES_OK;
    case NQES_OPT_TENSOR_CORES:
        if (value < 0 || value > 2) {
            ctx->err = "option value must be 0, 1 or 2";
            return NQES_ERR_INVALID;
        }
        ctx->tensor_cores = int(value);
        if (ctx->exec) {  // the captured step bakes the S·v kernels in
            cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
        }
        return NQES_OK;
    case NQES_OPT_MIXED_ENERGY64:
        if (value < 0 || value > 2) {
            ctx->err = "option value must be 0, 1 or 2";
            return NQES_ERR_INVALID;
        }
        ctx->mixed_e64 = int(value);
        if (ctx->exec) {  // the captured step bakes the sampler's arguments in
            cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
        }
        return NQES_OK;
    case NQES_OPT_TEST_STAGE_WAIT:
        if (value != 0 && value != 1) {
            ctx->err = "option value must be 0 or 1";
            return NQES_ERR_INVALID;
        }
        if (value == 1 && !ctx->dw_U) {
            ctx->err = "this shape has no staged sampler (the decision-warp form does not apply)";
            return NQES_ERR_INVALID;
        }
        ctx->stage_fault = int(value);
        if (ctx->exec) {  // the captured step bakes the sampler's arguments in
            cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
        }
        return NQES_OK;
    case NQES_OPT_FUSED_SV:
        if (value != -1 && value != 0 && value != 1) {
            ctx->err = "option value must be -1 (by precision), 0 or 1";
            return NQES_ERR_INVALID;
        }
        ctx->fused_opt = int(value);  // takes effect at the next step (the buffers are resized then)
        return NQES_OK;
    case NQES_OPT_SAMPLER_PLAN: {
        const int w = int(value & 15);
        if (value < 0 || value > 31 || (value != 0 && w != 1 && w != 2 && w != 4 && w != 8)) {
            ctx->err = "sampler plan must be 0, or 1, 2, 4 or 8 warps plus 16 for staged tables";
            return NQES_ERR_INVALID;
        }
        ctx->autotune = false;
        ctx->dw_force_warps = w;
        ctx->dw_force_stage = value >= 16 ? 1 : 0;
        if (ctx->exec) {  // the captured step bakes the sampler's launch in
            cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
        }
        return NQES_OK;
    }
    case NQES_OPT_REJECT_FILTER:
    case NQES_OPT_MIXED_EXACT:
        if (value != 0 && value != 1) {
            ctx->err = "option value must be 0 or 1";
            return NQES_ERR_INVALID;
        }
        if (option == NQES_OPT_REJECT_FILTER)
            ctx->reject_filter = value == 1;
        else
            ctx->mixed_exact_all = value == 1;
        if (ctx->exec) {  // the captured step bakes the sampler variant in
            cudaGraphExecDestroy(ctx->exec);
            ctx->exec = nullptr;
        }
        return NQES_OK;
    default:
        ctx->err = "unknown option " + std::to_string(option);
        return NQES_ERR_INVALID;
    }
}

int nqes_set_weights(nqes_ctx *ctx, const double *a, const double *b, const double *w) {
    if (!ctx || !a || !b || !w) return NQES_ERR_INVALID;
    const Shape &sh = ctx->sh;
    const bool real = host_weights_real(a, b, w, sh);
    if (ctx->arith_opt == NQES_ARITH_REAL && !real) {
        ctx->err = "weights have non-zero imaginary parts but arithmetic is forced REAL";
        return NQES_ERR_INVALID;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    NQES_CUDA(cudaMemcpyAsync(ctx->a, a, sizeof(cplx) * sh.K * sh.N, cudaMemcpyHostToDevice, ctx->st));
    NQES_CUDA(cudaMemcpyAsync(ctx->b, b, sizeof(cplx) * sh.K * sh.M, cudaMemcpyHostToDevice, ctx->st));
    NQES_CUDA(cudaMemcpyAsync(ctx->w, w, sizeof(cplx) * sh.K * sh.N * sh.M, cudaMemcpyHostToDevice, ctx->st));
    NQES_CUDA(cudaStreamSynchronize(ctx->st));
    ctx->weights_real = real;
    return NQES_OK;
}

int nqes_get_weights(nqes_ctx *ctx, double *a, double *b, double *w) {
    if (!ctx || !a || !b || !w) return NQES_ERR_INVALID;
    const Shape &sh = ctx->sh;
    NQES_CUDA(cudaSetDevice(ctx->device));
    NQES_CUDA(cudaMemcpyAsync(a, ctx->a, sizeof(cplx) * sh.K * sh.N, cudaMemcpyDeviceToHost, ctx->st));
    NQES_CUDA(cudaMemcpyAsync(b, ctx->b, sizeof(cplx) * sh.K * sh.M, cudaMemcpyDeviceToHost, ctx->st));
    NQES_CUDA(cudaMemcpyAsync(w, ctx->w, sizeof(cplx) * sh.K * sh.N * sh.M, cudaMemcpyDeviceToHost, ctx->st));
    NQES_CUDA(cudaStreamSynchronize(ctx->st));
    return NQES_OK;
}

int nqes_init_weights(nqes_ctx *ctx, uint64_t seed) {
    if (!ctx) return NQES_ERR_INVALID;
    // pcg64 as a UniformRandomBitGenerator for libstdc++'s normal_distribution.
    struct Urbg {
        using result_type = uint64_t;
        Pcg64 g;
        static constexpr uint64_t min() { return 0; }
        static constexpr uint64_t max() { return ~uint64_t(0); }
        uint64_t operator()() { return pcg_next(g); }
    } rg{pcg_seed(seed - 1)};
    const Shape &sh = ctx->sh;
    std::normal_distribution<double> nd;
    std::vector<double> a(2 * sh.K * sh.N), b(2 * sh.K * sh.M), w(2 * size_t(sh.K) * sh.N * sh.M);
    auto draw = [&](double *dst, double scale) {
        const double re = nd(rg), im = nd(rg);  // braced-init order of code/rbm.cc:248
        dst[0] = re / scale;
        dst[1] = im / scale;
    };
    for (int k = 0; k < sh.K; k++) {
        for (int i = 0; i < sh.N; i++) draw(&a[2 * (k * sh.N + i)], std::sqrt(double(sh.N)));
        for (int j = 0; j < sh.M; j++) draw(&b[2 * (k * sh.M + j)], std::sqrt(double(sh.M)));
        for (int i = 0; i < sh.N; i++)
            for (int j = 0; j < sh.M; j++)
                draw(&w[2 * ((size_t(k) * sh.N + i) * sh.M + j)], std::sqrt(double(sh.N * sh.M)));
    }
    return nqes_set_weights(ctx, a.data(), b.data(), w.data());
}

int nqes_sr_step(nqes_ctx *ctx, uint64_t seed, int chains, int m, int burn, double lr, double reglam, double rtol,
                 uint64_t maxit, double *e_mat, nqes_step_info *info) {
    if (!ctx) return NQES_ERR_INVALID;
    NvtxRange r_step("nqes_sr_step");
    int arith = 0;
    int rc;
    {
        NvtxRange r("prepare (arguments, buffers, autotune)");
        rc = step_prepare(ctx, seed, chains, m, burn, lr, reglam, rtol, maxit, &arith);
    }
    if (rc) return rc;
    {
        NvtxRange r("graph (capture when the shape changed) and launch");
        rc = arith == NQES_ARITH_COMPLEX ? sr_step_t<cplx>(ctx, chains, m, burn) : sr_step_t<double>(ctx, chains, m, burn);
    }
    if (rc) return rc;
    NvtxRange r_wait("device step and read-back");
    rc = step_readback(ctx, ctx->st);
    if (rc) return rc;
    NQES_CUDA(cudaStreamSynchronize(ctx->st));
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    return step_finish(ctx, chains, m, burn, arith, maxit, ms, e_mat, info);
}

int nqes_evaluate(nqes_ctx *ctx, const uint64_t *configs, int count, double *phi, double *tanh_theta, double *E,
                  double *O) {
    if (!ctx || !configs || count < 1) return NQES_ERR_INVALID;
    NQES_CUDA(cudaSetDevice(ctx->device));
    const Shape &sh = ctx->sh;
    const int arith = resolve_arith(ctx);
    const size_t KK = size_t(sh.K) * sh.K, ss = ssize(arith), words = size_t(count) * sh.K * sh.NW;
    uint64_t *cfg = nullptr, *sp = nullptr;
    cplx *dphi = nullptr, *dth = nullptr, *dE = nullptr, *ddm = nullptr;
    unsigned char *dO = nullptr;
    int rc;
    if ((rc = dalloc(ctx, &cfg, words)) || (rc = dalloc(ctx, &sp, words)) || (rc = dalloc(ctx, &dphi, count * KK)) ||
        (rc = dalloc(ctx, &dth, count * KK * sh.M)) || (rc = dalloc(ctx, &dE, count * KK)) ||
        (rc = dalloc(ctx, &ddm, count * KK)) || (rc = dalloc(ctx, &dO, size_t(count) * sh.P * ss))) {
        dfree(cfg); dfree(sp); dfree(dphi); dfree(dth); dfree(dE); dfree(ddm); dfree(dO);
        return rc;
    }
    int status = NQES_OK;
    auto run = [&]() -> int {
        NQES_CUDA(cudaMemcpy(cfg, configs, words * 8, cudaMemcpyHostToDevice));
        NQES_CUDA(cudaMemset(ctx->err_d, 0, sizeof(int)));
        const int tk = choose_tk(ctx, count);
        if (arith == NQES_ARITH_COMPLEX) {
            NQES_CUDA(prepare_sample<cplx>(sh));
            NQES_CUDA(launch_tables_ctx<cplx>(ctx));
            SampleArgs<cplx> A = sample_args<cplx>(ctx, count, 1, 0, tk);
            A.O = reinterpret_cast<cplx *>(dO);
            A.E = dE;
            A.spins = sp;
            A.cfg = cfg;
            A.phi_out = dphi;
            A.tanh_out = dth;
            A.dm_out = ddm;
            NQES_CUDA(launch_sample<cplx>(A, sample_threads(sh.K, tk), ctx->st));
        } else {
            NQES_CUDA(prepare_sample<double>(sh));
            NQES_CUDA(launch_tables_ctx<double>(ctx));
            SampleArgs<double> A = sample_args<double>(ctx, count, 1, 0, tk);
            A.O = reinterpret_cast<double *>(dO);
            A.E = dE;
            A.spins = sp;
            A.cfg = cfg;
            A.phi_out = dphi;
            A.tanh_out = dth;
            A.dm_out = ddm;
            NQES_CUDA(launch_sample<double>(A, sample_threads(sh.K, tk), ctx->st));
        }
        NQES_CUDA(launch_eval_singular(count, sh.K, dphi, ddm, dE, reinterpret_cast<double *>(dO),
                                       size_t(sh.P) * ss / sizeof(double), ctx->st));
        NQES_CUDA(cudaStreamSynchronize(ctx->st));
        if (phi) NQES_CUDA(cudaMemcpy(phi, dphi, count * KK * sizeof(cplx), cudaMemcpyDeviceToHost));
        if (tanh_theta) NQES_CUDA(cudaMemcpy(tanh_theta, dth, count * KK * sh.M * sizeof(cplx), cudaMemcpyDeviceToHost));
        if (E) NQES_CUDA(cudaMemcpy(E, dE, count * KK * sizeof(cplx), cudaMemcpyDeviceToHost));
        if (O) {
            const int saved = ctx->arith;
            ctx->arith = arith;
            int r = copy_out_c(ctx, dO, size_t(count) * sh.P, O);
            ctx->arith = saved;
            if (r) return r;
        }
        int e = 0;
        NQES_CUDA(cudaMemcpy(&e, ctx->err_d, sizeof(int), cudaMemcpyDeviceToHost));
        e &= ~int(kErrSingular);  // rank-deficient Phi: E and O come from k_eval_singular
        if (e) {
            ctx->err = "evaluation flagged error bits " + std::to_string(e);
            return NQES_ERR_NONFINITE;
        }
        return NQES_OK;
    };
    status = run();
    dfree(cfg); dfree(sp); dfree(dphi); dfree(dth); dfree(dE); dfree(ddm); dfree(dO);
    return status;
}

int nqes_get_samples(nqes_ctx *ctx, uint64_t *configs, double *eloc, double *E) {
    if (!ctx) return NQES_ERR_INVALID;
    if (!ctx->have_step) {
        ctx->err = "no SR step has run";
        return NQES_ERR_STATE;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    const size_t KK = size_t(ctx->sh.K) * ctx->sh.K;
    if (configs)
        NQES_CUDA(cudaMemcpy(configs, ctx->spins, ctx->Ns * ctx->sh.K * ctx->sh.NW * 8, cudaMemcpyDeviceToHost));
    if (eloc || E) {
        std::vector<cplx> e(ctx->Ns * KK);
        NQES_CUDA(cudaMemcpy(e.data(), ctx->E, e.size() * sizeof(cplx), cudaMemcpyDeviceToHost));
        if (E) std::memcpy(E, e.data(), e.size() * sizeof(cplx));
        if (eloc)
            for (size_t s = 0; s < ctx->Ns; s++) {
                cplx t{0, 0};
                for (int k = 0; k < ctx->sh.K; k++) t += e[s * KK + k * ctx->sh.K + k];
                eloc[2 * s] = t.re;
                eloc[2 * s + 1] = t.im;
            }
    }
    return NQES_OK;
}

int nqes_get_accepts(nqes_ctx *ctx, uint64_t *accepted) {
    if (!ctx || !accepted) return NQES_ERR_INVALID;
    if (!ctx->have_step) {
        ctx->err = "no SR step has run";
        return NQES_ERR_STATE;
    }
    NQES_CUDA(cudaMemcpy(accepted, ctx->accepted, sizeof(uint64_t) * ctx->chains, cudaMemcpyDeviceToHost));
    return NQES_OK;
}

int nqes_get_O(nqes_ctx *ctx, int first, int count, double *O) {
    if (!ctx || !O || first < 0 || count < 1) return NQES_ERR_INVALID;
    if (!ctx->have_step || size_t(first) + count > ctx->Ns) {
        ctx->err = "rows out of range or no SR step has run";
        return NQES_ERR_STATE;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    const size_t P = ctx->sh.P;
    if (ctx->step_precision == NQES_PRECISION_MIXED) {
        // the rows rebuilt from the factors the mixed form keeps
        std::vector<float> tmp(size_t(count) * P);
        float *d = nullptr;
        NQES_CUDA(cudaMalloc(&d, tmp.size() * sizeof(float)));
        cudaError_t e = launch_fO(fact_args(ctx), first, count, d, ctx->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(tmp.data(), d, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        cudaFree(d);
        if (e != cudaSuccess) {
            ctx->err = cudaGetErrorString(e);
            return NQES_ERR_CUDA;
        }
        for (size_t t = 0; t < tmp.size(); t++) {
            O[2 * t] = tmp[t];
            O[2 * t + 1] = 0.0;
        }
        return NQES_OK;
    }
    const unsigned char *src = static_cast<const unsigned char *>(ctx->O) + size_t(first) * P * ssize(ctx->arith);
    if (o_split(ctx)) {  // stored as double-float pairs: hi + lo
        std::vector<float> tmp(2 * size_t(count) * P);
        NQES_CUDA(cudaMemcpyAsync(tmp.data(), src, tmp.size() * sizeof(float), cudaMemcpyDeviceToHost, ctx->st));
        NQES_CUDA(cudaStreamSynchronize(ctx->st));
        for (size_t t = 0; t < size_t(count) * P; t++) {
            O[2 * t] = double(tmp[2 * t]) + double(tmp[2 * t + 1]);
            O[2 * t + 1] = 0.0;
        }
        return NQES_OK;
    }
    return copy_out_c(ctx, src, size_t(count) * P, O);
}

int nqes_get_moments(nqes_ctx *ctx, double *o, double *skk, double *f) {
    if (!ctx) return NQES_ERR_INVALID;
    if (!ctx->have_step) {
        ctx->err = "no SR step has run";
        return NQES_ERR_STATE;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    const size_t P = ctx->sh.P, ss = ssize(ctx->arith);
    const unsigned char *v = static_cast<const unsigned char *>(ctx->vecs);
    int rc;
    if (o && (rc = copy_out_c(ctx, v + 0 * P * ss, P, o))) return rc;
    if (skk && (rc = copy_out_c(ctx, v + 1 * P * ss, P, skk))) return rc;
    if (f && (rc = copy_out_c(ctx, v + 2 * P * ss, P, f))) return rc;
    return NQES_OK;
}

int nqes_get_solution(nqes_ctx *ctx, double *x) {
    if (!ctx || !x) return NQES_ERR_INVALID;
    if (!ctx->have_step) {
        ctx->err = "no SR step has run";
        return NQES_ERR_STATE;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    const size_t P = ctx->sh.P, ss = ssize(ctx->arith);
    return copy_out_c(ctx, static_cast<const unsigned char *>(ctx->vecs) + 11 * P * ss, P, x);
}

int nqes_apply_S(nqes_ctx *ctx, const double *v, double *out) {
    if (!ctx || !v || !out) return NQES_ERR_INVALID;
    if (!ctx->have_step) {
        ctx->err = "no SR step has run";
        return NQES_ERR_STATE;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    const size_t P = ctx->sh.P, ss = ssize(ctx->arith);
    unsigned char *dv = nullptr, *dout = nullptr;
    int rc;
    if ((rc = dalloc(ctx, &dv, P * ss)) || (rc = dalloc(ctx, &dout, P * ss))) {
        dfree(dv);
        return rc;
    }
    auto run = [&]() -> int {
        if (ctx->arith == NQES_ARITH_COMPLEX) {
            NQES_CUDA(cudaMemcpy(dv, v, P * sizeof(cplx), cudaMemcpyHostToDevice));
            SolveBufs<cplx> B = solve_bufs<cplx>(ctx);
            NQES_CUDA(launch_apply_S<cplx>(B, reinterpret_cast<cplx *>(dv), reinterpret_cast<cplx *>(dout), ctx->st));
        } else {
            std::vector<double> tmp(P);
            for (size_t t = 0; t < P; t++) tmp[t] = v[2 * t];
            NQES_CUDA(cudaMemcpy(dv, tmp.data(), P * sizeof(double), cudaMemcpyHostToDevice));
            SolveBufs<double> B = solve_bufs<double>(ctx);
            if (B.fact) NQES_CUDA(prepare_mixed_sampler(ctx));
            NQES_CUDA(launch_apply_S<double>(B, reinterpret_cast<double *>(dv), reinterpret_cast<double *>(dout),
                                             ctx->st));
        }
        NQES_CUDA(cudaStreamSynchronize(ctx->st));
        return copy_out_c(ctx, dout, P, out);
    };
    rc = run();
    dfree(dv);
    dfree(dout);
    return rc;
}

}  // extern "C"

namespace {
template <class S> int time_kernel_t(nqes_ctx *ctx, int kernel, int reps, double *avg_ms, double *bytes) {
    SolveBufs<S> B = solve_bufs<S>(ctx);
    const size_t Ns = ctx->Ns, P = ctx->sh.P, ss = sizeof(S), KK = size_t(ctx->sh.K) * ctx->sh.K;
    auto launch = [&]() -> cudaError_t {
        switch (kernel) {
        case NQES_KERNEL_SAMPLE: {
            if (uses_mixed_sampler(ctx))
                return launch_mixed_sampler(ctx, ctx->chains, ctx->m, ctx->last_burn, ctx->last_tk);
            SampleArgs<S> A = sample_args<S>(ctx, ctx->chains, ctx->m, ctx->last_burn, ctx->last_tk);
            return launch_sample<S>(A, sample_threads(ctx->sh.K, ctx->last_tk), ctx->st);
        }
        case NQES_KERNEL_SV_ROWS:
        case NQES_KERNEL_SV_COLS:
            if (B.o_split) return cudaErrorNotSupported;  // the two-pass kernels read FP64 entries
            return kernel == NQES_KERNEL_SV_ROWS ? launch_sv_rows_only<S>(B, ctx->st) : launch_sv_cols_only<S>(B, ctx->st);
        case NQES_KERNEL_SV: return launch_sv_only<S>(B, ctx->st);
        default: return launch_moment_part_only<S>(B, ctx->st);
        }
    };
    switch (kernel) {
    case NQES_KERNEL_SAMPLE: *bytes = double(Ns) * (P * ss + KK * sizeof(cplx) + ctx->sh.K * ctx->sh.NW * 8); break;
    case NQES_KERNEL_SV_ROWS: *bytes = double(Ns) * P * ss + double(P) * ss + double(Ns) * ss; break;
    case NQES_KERNEL_SV_COLS: *bytes = double(Ns) * P * ss + double(Ns) * ss + double(ctx->rchunks) * P * ss; break;
    case NQES_KERNEL_SV:  // fused: O once, v, one partial per CTA; two-pass: both passes
        *bytes = B.fG ? double(Ns) * P * ss + double(P) * ss + double(B.svp) * P * ss
                      : 2.0 * double(Ns) * P * ss + double(P) * ss + 2.0 * double(Ns) * ss + double(ctx->rchunks) * P * ss;
        break;
    default: *bytes = double(Ns) * P * ss + double(Ns) * KK * sizeof(cplx) + 3.0 * ctx->rchunks * P * ss; break;
    }
    const bool mixed = ctx->step_precision == NQES_PRECISION_MIXED;
    if (mixed) {
        // the factors of O: K^2 (M + 1) floats per sample, plus the spins for the signs
        const double fac = double(Ns) * (double(KK) * (ctx->sh.M + 1) * 4 + ctx->sh.K * ctx->sh.NW * 8);
        switch (kernel) {
        case NQES_KERNEL_SAMPLE: *bytes = fac + double(Ns) * KK * sizeof(cplx); break;
        case NQES_KERNEL_SV_ROWS: *bytes = fac + double(P) * 4 + double(Ns) * 4; break;
        case NQES_KERNEL_SV_COLS: *bytes = fac + double(Ns) * 4 + double(ctx->rchunks) * P * 4; break;
        case NQES_KERNEL_SV: *bytes = 2.0 * fac + double(P) * 4 + 2.0 * double(Ns) * 4 + double(ctx->rchunks) * P * 4; break;
        default: *bytes = fac + double(Ns) * KK * sizeof(cplx) + 3.0 * ctx->rchunks * P * 4; break;
        }
        NQES_CUDA(prepare_mixed_sampler(ctx));
    }
    if (kernel == NQES_KERNEL_SAMPLE) {
        if (uses_mixed_sampler(ctx))
            NQES_CUDA(prepare_mixed_sampler(ctx));
        else
            NQES_CUDA(prepare_sample<S>(ctx->sh));
    }
    NQES_CUDA(launch());  // warm-up
    NQES_CUDA(cudaStreamSynchronize(ctx->st));
    NQES_CUDA(cudaEventRecord(ctx->ev0, ctx->st));
    for (int r = 0; r < reps; r++) NQES_CUDA(launch());
    NQES_CUDA(cudaEventRecord(ctx->ev1, ctx->st));
    NQES_CUDA(cudaEventSynchronize(ctx->ev1));
    float ms = 0;
    NQES_CUDA(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    *avg_ms = double(ms) / reps;
    return NQES_OK;
}
}  // namespace

extern "C" {

int nqes_time_kernel(nqes_ctx *ctx, int kernel, int reps, double *avg_ms, double *algorithmic_bytes) {
    if (!ctx || !avg_ms || !algorithmic_bytes || reps < 1 || kernel < NQES_KERNEL_SAMPLE || kernel > NQES_KERNEL_SV)
        return NQES_ERR_INVALID;
    if (!ctx->have_step) {
        ctx->err = "no SR step has run";
        return NQES_ERR_STATE;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    return ctx->arith == NQES_ARITH_COMPLEX ? time_kernel_t<cplx>(ctx, kernel, reps, avg_ms, algorithmic_bytes)
                                            : time_kernel_t<double>(ctx, kernel, reps, avg_ms, algorithmic_bytes);
}

}  // extern "C"

namespace {
template <class S>
int correlations_t(nqes_ctx *ctx, uint64_t seed, int chains, int m, int burn, const cplx *evecs, double *x, double *z,
                   double *xx, double *zz) {
    const Shape &sh = ctx->sh;
    const int N = sh.N, K = sh.K, KK = K * K;
    const size_t stride = 2 * size_t(N) * KK + 2 * size_t(N) * N * KK;
    S *acc = nullptr, *scratch = nullptr, *out = nullptr;
    uint64_t *spins = nullptr;
    int rc;
    if ((rc = dalloc(ctx, &acc, size_t(chains) * stride)) ||
        (rc = dalloc(ctx, &scratch, size_t(chains) * N * N * KK)) || (rc = dalloc(ctx, &out, stride)) ||
        (rc = dalloc(ctx, &spins, size_t(chains) * m * K * sh.NW))) {
        dfree(acc); dfree(scratch); dfree(out); dfree(spins);
        return rc;
    }
    auto run = [&]() -> int {
        StepParams p{};
        p.seed = seed;
        NQES_CUDA(cudaMemcpyAsync(ctx->sp, &p, sizeof(p), cudaMemcpyHostToDevice, ctx->st));
        NQES_CUDA(cudaMemsetAsync(acc, 0, sizeof(S) * chains * stride, ctx->st));
        NQES_CUDA(cudaMemsetAsync(ctx->err_d, 0, sizeof(int), ctx->st));
        NQES_CUDA(prepare_sample<S>(sh));
        NQES_CUDA(launch_tables_ctx<S>(ctx));
        const int tk = choose_tk(ctx, chains);
        SampleArgs<S> A = sample_args<S>(ctx, chains, m, burn, tk);
        A.O = nullptr;
        A.E = nullptr;
        A.spins = spins;
        A.accepted = nullptr;
        A.corr = acc;
        A.corr_scratch = scratch;
        A.corr_stride = stride;
        NQES_CUDA(launch_sample<S>(A, sample_threads(K, tk), ctx->st));
        NQES_CUDA(launch_corr_reduce<S>(acc, chains, stride, out, ctx->st));
        std::vector<S> h(stride);
        NQES_CUDA(cudaMemcpyAsync(h.data(), out, sizeof(S) * stride, cudaMemcpyDeviceToHost, ctx->st));
        int e = 0;
        NQES_CUDA(cudaMemcpyAsync(&e, ctx->err_d, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        NQES_CUDA(cudaStreamSynchronize(ctx->st));
        // res(i, k) = Re diag(V^-1 (sum_i / Ns) V)_k  (code/rbm.cc:761-769)
        cplx vinv[16];
        if (!small_inv(evecs, vinv, K)) {
            ctx->err = "eigenvector matrix is singular";
            return NQES_ERR_INVALID;
        }
        const double ns = double(chains) * m;
        auto finish = [&](size_t off, size_t rows, double *dst) {
            for (size_t r = 0; r < rows; r++) {
                cplx mat[16], t1[16];
                for (int q = 0; q < KK; q++) mat[q] = to_c(h[off + r * KK + q]) * (1.0 / ns);
                for (int a = 0; a < K; a++)
                    for (int b = 0; b < K; b++) {
                        cplx s{0, 0};
                        for (int t = 0; t < K; t++) s += vinv[a * K + t] * mat[t * K + b];
                        t1[a * K + b] = s;
                    }
                for (int k = 0; k < K; k++) {
                    cplx s{0, 0};
                    for (int t = 0; t < K; t++) s += t1[k * K + t] * evecs[t * K + k];
                    dst[r * K + k] = s.re;
                }
            }
        };
        finish(0, N, x);
        finish(size_t(N) * KK, N, z);
        finish(2 * size_t(N) * KK, size_t(N) * N, xx);
        finish(2 * size_t(N) * KK + size_t(N) * N * KK, size_t(N) * N, zz);
        if (e & (kErrNonFinite | kErrSingular)) {
            ctx->err = "non-finite value or singular Phi in the correlation pass (error bits " + std::to_string(e) + ")";
            return NQES_ERR_NONFINITE;
        }
        return NQES_OK;
    };
    rc = run();
    dfree(acc); dfree(scratch); dfree(out); dfree(spins);
    return rc;
}
}  // namespace

extern "C" {

int nqes_correlations(nqes_ctx *ctx, uint64_t seed, int chains, int m, int burn, const double *evecs, double *x,
                      double *z, double *xx, double *zz) {
    if (!ctx || !evecs || !x || !z || !xx || !zz || chains < 1 || m < 1 || burn < 0) {
        if (ctx) ctx->err = "invalid correlation arguments";
        return NQES_ERR_INVALID;
    }
    NQES_CUDA(cudaSetDevice(ctx->device));
    const int arith = resolve_arith(ctx);
    const cplx *V = reinterpret_cast<const cplx *>(evecs);
    return arith == NQES_ARITH_COMPLEX ? correlations_t<cplx>(ctx, seed, chains, m, burn, V, x, z, xx, zz)
                                       : correlations_t<double>(ctx, seed, chains, m, burn, V, x, z, xx, zz);
}

}  // extern "C"

extern "C" int nqes_footprint_bytes(int n_spins, int n_hidden, int n_states, int chains, int samples_per_chain,
                                    int precision, int complex_arith, uint64_t *bytes) {
    if (!bytes || n_spins < 1 || n_hidden < 1 || n_states < 1 || chains < 1 || samples_per_chain < 1)
        return NQES_ERR_INVALID;
    const uint64_t N = n_spins, M = n_hidden, K = n_states, NW = (N + 63) / 64, P = K * (N + M + N * M);
    const uint64_t Ns = uint64_t(chains) * samples_per_chain, ss = complex_arith ? 16 : 8;
    const bool mixed = precision == NQES_PRECISION_MIXED;
    const uint64_t rchunks = 32, nw = K * N * M, na = K * N;
    uint64_t b = mixed ? Ns * K * K * (((M + 3) & ~3ULL) + 1) * 4 : Ns * P * ss;  // O, or its factors (mixed)
    b += Ns * K * K * 16 + Ns * K * NW * 8 + uint64_t(chains) * 16;  // E, spins, accept / exact counts
    b += Ns * ss + 3 * rchunks * P * ss + 16 * P * ss + 4 * kPartStride * 8;
    if (mixed) b += P * 4 + Ns * 4 + 3 * 256 * P * 4;
    b += (3 * nw + 2 * na + K * M) * 16 + N * N * 8;  // weights, FP64 tables (complex-sized), J
    b += nw * 4 * 2 + na * 4 * 2 + (nw + na + K * M) * 8;  // FP32 tables and FP64 copies of the real weights
    b += 6 * K * N * 512 * 4 + 6 * K * 512 * 4 + (4 * K * N + 4 * K) * 4;  // decision-warp tables (upper bound)
    *bytes = b + (uint64_t(4) << 20);                        // small buffers and allocation rounding
    return NQES_OK;
}

// ---- batched multi-solve ----

struct nqes_batch {
    std::vector<nqes_ctx *> m;
    int device = 0;
    cudaStream_t st = nullptr;
    cudaStream_t sq = nullptr;          // the loop body's QLP branch (capture only)
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEvent_t ev_fork = nullptr;      // fork of the loop body's branches (capture only)
    cudaEvent_t ev_qjoin = nullptr;     // join of the QLP branch (capture only)
    const int **flags_d = nullptr;      // device array: each member's QlpState::running
    void *groups_d = nullptr;           // the loop body's grouped-launch tables (see the capture)
    cudaGraphExec_t exec = nullptr;
    std::vector<std::vector<long long>> keys;  // per member: what its captured nodes depend on (see the step)
    std::string err;
};

namespace {
thread_local std::string g_batch_create_error;

// The loop body of a batch as grouped launches (one launch per kernel for all
// the members it covers, kernels_solve.cu / kernels_factored.cu): the members'
// buffers as device tables, in member order per arithmetic, and the factored
// S·v passes of the MIXED members grouped by kernel variant. Members whose S·v
// has no grouped form (two-pass or fused FP64 S·v, tensor-core passes) run it
// with their own launches on their own streams. Each member's arithmetic is
// that of its own loop body.
struct FactGroup {
    int variant = 0, blocks = 0;
    size_t smem = 0;
    std::vector<FactMember> mem;
    std::vector<int> first{0};
    size_t off_tab = 0, off_first = 0;  // byte offsets in groups_d
};
struct BodyGroups {
    std::vector<SolveBufs<double>> tabd;
    std::vector<SolveBufs<cplx>> tabc;
    std::vector<int> firstd{0}, firstc{0};
    size_t off_tabd = 0, off_tabc = 0, off_firstd = 0, off_firstc = 0;
    std::vector<FactGroup> rows, cols;
    std::vector<int> own_rows;  // members that run their rows pass (or whole S·v) on their own stream
    std::vector<int> own_cols;  // MIXED members that run their column pass on their own stream
};

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

FactGroup &group_of(std::vector<FactGroup> &v, int variant) {
    for (auto &g : v)
        if (g.variant == variant) return g;
    v.emplace_back();
    v.back().variant = variant;
    return v.back();
}

// Builds the tables (host side), uploads them to b->groups_d and sets the
// grouped kernels' shared-memory limits (not allowed during a capture).
int plan_body_groups(nqes_batch *b, const std::vector<int> &arith, BodyGroups &g) {
    const int n = int(b->m.size());
    for (int i = 0; i < n; i++) {
        nqes_ctx *c = b->m[i];
        const int *guard = running_flag(c);
        if (arith[i] == NQES_ARITH_COMPLEX) {
            SolveBufs<cplx> B = solve_bufs<cplx>(c);
            B.use_cond = 0;
            B.guard = guard;
            g.tabc.push_back(B);
            g.firstc.push_back(g.firstc.back() + minres_vector_blocks(c->sh.P));
            g.own_rows.push_back(i);
            continue;
        }
        SolveBufs<double> B = solve_bufs<double>(c);
        B.use_cond = 0;
        B.guard = guard;
        B.F.guard = guard;
        g.tabd.push_back(B);
        g.firstd.push_back(g.firstd.back() + minres_vector_blocks(c->sh.P));
        if (!B.fact) {
            g.own_rows.push_back(i);
            continue;
        }
        const FactGroupPlan pl = fact_group_plan(B.F);
        FactMember fm{};
        fm.F = B.F;
        fm.F.ic = pl.ic;
        fm.v32 = B.v32;
        fm.u32 = B.u32;
        fm.ypart32 = B.ypart32;
        fm.gn = pl.gn;
        fm.zg = pl.zg;
        const cudaError_t pe = prepare_fact_group(pl);
        if (pe != cudaSuccess) {
            b->err = std::string("grouped S·v kernels: ") + cudaGetErrorString(pe);
            return NQES_ERR_CUDA;
        }
        if (B.F.tc) {
            g.own_rows.push_back(i);
        } else {
            FactGroup &r = group_of(g.rows, pl.rows_variant);
            r.mem.push_back(fm);
            r.blocks += pl.rows_blocks;
            r.first.push_back(r.blocks);
            r.smem = std::max(r.smem, pl.rows_smem);
        }
        if (B.F.tcc) {
            g.own_cols.push_back(i);
        } else {
            FactGroup &q = group_of(g.cols, pl.cols_variant);
            q.mem.push_back(fm);
            q.blocks += pl.cols_blocks;
            q.first.push_back(q.blocks);
            q.smem = std::max(q.smem, pl.cols_smem);
        }
    }
    // Rows groups of variant 2 (4 j-threads x 16 columns, 2 rows a group: the
    // latency form of one solve) with more than two waves of blocks take 4
    // rows a group (variant 6): the same per-row arithmetic in half the blocks.
    for (FactGroup &r : g.rows) {
        if (r.variant != 2 || r.blocks <= 6 * 152) continue;
        r.variant = 6;
        r.blocks = 0;
        r.smem = 0;
        r.first.assign(1, 0);
        for (const FactMember &fm : r.mem) {
            int blocks = 0, ic = 0;
            size_t smem = 0;
            fact_rows_geometry(6, fm.F, &blocks, &smem, &ic);
            r.blocks += blocks;
            r.first.push_back(r.blocks);
            r.smem = std::max(r.smem, smem);
        }
        FactGroupPlan pl{};
        pl.rows_variant = 6;
        pl.cols_variant = fact_group_plan(r.mem[0].F).cols_variant;
        const cudaError_t pe = prepare_fact_group(pl);
        if (pe != cudaSuccess) {
            b->err = std::string("grouped S·v kernels: ") + cudaGetErrorString(pe);
            return NQES_ERR_CUDA;
        }
    }
    // one device buffer for every table
    size_t off = 0;
    auto place = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes);
        return o;
    };
    g.off_tabd = place(g.tabd.size() * sizeof(SolveBufs<double>));
    g.off_tabc = place(g.tabc.size() * sizeof(SolveBufs<cplx>));
    g.off_firstd = place(g.firstd.size() * sizeof(int));
    g.off_firstc = place(g.firstc.size() * sizeof(int));
    for (auto *v : {&g.rows, &g.cols})
        for (auto &fg : *v) {
            fg.off_tab = place(fg.mem.size() * sizeof(FactMember));
            fg.off_first = place(fg.first.size() * sizeof(int));
        }
    std::vector<unsigned char> host(std::max<size_t>(off, 256));
    auto put = [&](size_t o, const void *src, size_t bytes) {
        if (bytes) std::memcpy(host.data() + o, src, bytes);
    };
    put(g.off_tabd, g.tabd.data(), g.tabd.size() * sizeof(SolveBufs<double>));
    put(g.off_tabc, g.tabc.data(), g.tabc.size() * sizeof(SolveBufs<cplx>));
    put(g.off_firstd, g.firstd.data(), g.firstd.size() * sizeof(int));
    put(g.off_firstc, g.firstc.data(), g.firstc.size() * sizeof(int));
    for (auto *v : {&g.rows, &g.cols})
        for (auto &fg : *v) {
            put(fg.off_tab, fg.mem.data(), fg.mem.size() * sizeof(FactMember));
            put(fg.off_first, fg.first.data(), fg.first.size() * sizeof(int));
        }
    if (b->groups_d) {  // the previous graph, which used it, is destroyed and idle
        cudaFree(b->groups_d);
        b->groups_d = nullptr;
    }
    if (cudaMalloc(&b->groups_d, host.size()) != cudaSuccess ||
        cudaMemcpy(b->groups_d, host.data(), host.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        b->err = "allocation of the batch's launch tables failed";
        return NQES_ERR_OOM;
    }
    return NQES_OK;
}

// Captures the loop body onto b->st (in capture): the QLP branch of every
// member (grouped, on b->sq) beside the Lanczos branch (the S·v passes, then
// the grouped Lanczos kernels), joined on b->st.
cudaError_t capture_grouped_body(nqes_batch *b, const BodyGroups &g) {
    unsigned char *base = static_cast<unsigned char *>(b->groups_d);
    const auto *tabd = reinterpret_cast<const SolveBufs<double> *>(base + g.off_tabd);
    const auto *tabc = reinterpret_cast<const SolveBufs<cplx> *>(base + g.off_tabc);
    const int *firstd = reinterpret_cast<const int *>(base + g.off_firstd);
    const int *firstc = reinterpret_cast<const int *>(base + g.off_firstc);
    const int nd = int(g.tabd.size()), nc = int(g.tabc.size());
    cudaError_t e = cudaEventRecord(b->ev_fork, b->st);
    // QLP branch
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->sq, b->ev_fork, 0);
    if (e == cudaSuccess && nd) e = launch_qlp_group<double>(tabd, firstd, nd, g.firstd.back(), b->sq);
    if (e == cudaSuccess && nc) e = launch_qlp_group<cplx>(tabc, firstc, nc, g.firstc.back(), b->sq);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev_qjoin, b->sq);
    // Lanczos branch: members with their own S·v launches on their own streams
    for (int i : g.own_rows) {
        if (e != cudaSuccess) break;
        nqes_ctx *c = b->m[i];
        e = cudaStreamWaitEvent(c->st, b->ev_fork, 0);
        if (e != cudaSuccess) break;
        if (c->arith == NQES_ARITH_COMPLEX) {
            SolveBufs<cplx> B = solve_bufs<cplx>(c);
            B.use_cond = 0;
            B.guard = running_flag(c);
            e = launch_sv_only<cplx>(B, c->st);
        } else {
            SolveBufs<double> B = solve_bufs<double>(c);
            B.use_cond = 0;
            B.guard = running_flag(c);
            B.F.guard = B.guard;
            e = B.fact ? launch_sv_rows_only<double>(B, c->st) : launch_sv_only<double>(B, c->st);
        }
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_join, c->st);
    }
    for (const FactGroup &fg : g.rows) {
        if (e != cudaSuccess) break;
        e = launch_frows_group(fg.variant, reinterpret_cast<const FactMember *>(base + fg.off_tab),
                               reinterpret_cast<const int *>(base + fg.off_first), int(fg.mem.size()), fg.blocks,
                               fg.smem, b->st);
    }
    for (int i : g.own_rows)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->m[i]->ev_join, 0);
    // column passes after every rows pass (a member's rows may have run on its own stream)
    for (int i : g.own_cols) {
        if (e != cudaSuccess) break;
        nqes_ctx *c = b->m[i];
        SolveBufs<double> B = solve_bufs<double>(c);
        B.use_cond = 0;
        B.guard = running_flag(c);
        B.F.guard = B.guard;
        e = cudaEventRecord(c->ev_fork, b->st);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->st, c->ev_fork, 0);
        if (e == cudaSuccess) e = launch_sv_cols_only<double>(B, c->st);
        if (e == cudaSuccess) e = cudaEventRecord(c->ev_join, c->st);
    }
    for (const FactGroup &fg : g.cols) {
        if (e != cudaSuccess) break;
        e = launch_fcols_group(fg.variant, reinterpret_cast<const FactMember *>(base + fg.off_tab),
                               reinterpret_cast<const int *>(base + fg.off_first), int(fg.mem.size()), fg.blocks,
                               fg.smem, b->st);
    }
    for (int i : g.own_cols)
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->m[i]->ev_join, 0);
    // the Lanczos kernels of every member, then the join of the QLP branch
    if (e == cudaSuccess && nd) e = launch_lanczos_group<double>(tabd, firstd, nd, g.firstd.back(), b->st);
    if (e == cudaSuccess && nc) e = launch_lanczos_group<cplx>(tabc, firstc, nc, g.firstc.back(), b->st);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->ev_qjoin, 0);
    return e;
}
}  // namespace

extern "C" {

const char *nqes_batch_last_error(const nqes_batch *b) { return b ? b->err.c_str() : g_batch_create_error.c_str(); }

int nqes_batch_create(nqes_ctx *const *members, int count, nqes_batch **out) {
    if (!out || !members || count < 1) {
        g_batch_create_error = "members and out must be non-NULL and count >= 1";
        return NQES_ERR_INVALID;
    }
    *out = nullptr;
    for (int i = 0; i < count; i++) {
        if (!members[i]) {
            g_batch_create_error = "member " + std::to_string(i) + " is NULL";
            return NQES_ERR_INVALID;
        }
        if (members[i]->device != members[0]->device) {
            g_batch_create_error = "members live on different devices";
            return NQES_ERR_INVALID;
        }
        for (int j = 0; j < i; j++)
            if (members[j] == members[i]) {
                g_batch_create_error = "a context appears twice in the batch";
                return NQES_ERR_INVALID;
            }
    }
    nqes_batch *b = new nqes_batch();
    b->m.assign(members, members + count);
    b->device = members[0]->device;
    if (cudaSetDevice(b->device) != cudaSuccess || cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->sq, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_qjoin, cudaEventDisableTiming) != cudaSuccess) {
        g_batch_create_error = "stream or event creation failed";
        nqes_batch_destroy(b);
        return NQES_ERR_CUDA;
    }
    std::vector<const int *> flags(count);
    for (int i = 0; i < count; i++) flags[i] = running_flag(members[i]);
    if (cudaMalloc(reinterpret_cast<void **>(&b->flags_d), sizeof(int *) * count) != cudaSuccess ||
        cudaMemcpy(b->flags_d, flags.data(), sizeof(int *) * count, cudaMemcpyHostToDevice) != cudaSuccess) {
        g_batch_create_error = "allocation of the batch's flag table failed";
        nqes_batch_destroy(b);
        return NQES_ERR_OOM;
    }
    *out = b;
    return NQES_OK;
}

int nqes_batch_destroy(nqes_batch *b) {
    if (!b) return NQES_OK;
    cudaSetDevice(b->device);
    if (b->st) cudaStreamSynchronize(b->st);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->flags_d) cudaFree(b->flags_d);
    if (b->groups_d) cudaFree(b->groups_d);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_qjoin) cudaEventDestroy(b->ev_qjoin);
    if (b->sq) cudaStreamDestroy(b->sq);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return NQES_OK;
}

int nqes_batch_sr_step(nqes_batch *b, const uint64_t *seeds, const int *chains, const int *samples, const int *burn,
                       const double *lr, const double *reglam, const double *rtol, const uint64_t *maxit,
                       double *const *e_mats, nqes_step_info *infos, int *statuses, double *ms_total) {
    if (!b || !seeds || !chains || !samples || !burn || !lr || !reglam || !rtol || !maxit) return NQES_ERR_INVALID;
    NvtxRange r_step("nqes_batch_sr_step");
    const int n = int(b->m.size());
    if (cudaSetDevice(b->device) != cudaSuccess) {
        b->err = "cudaSetDevice failed";
        return NQES_ERR_CUDA;
    }
    std::vector<int> arith(n), tks(n);
    std::vector<std::vector<long long>> keys(n);
    if (statuses)
        for (int i = 0; i < n; i++) statuses[i] = NQES_ERR_STATE;  // not run (yet)
    // The members' samplers share the GPU: plan their launch shapes for the
    // chains of the whole batch (reset when this call returns).
    long long total = 0;
    for (int i = 0; i < n; i++) total += std::max(0, chains[i]);
    struct PlanScope {
        std::vector<nqes_ctx *> &m;
        ~PlanScope() {
            for (auto *c : m) c->plan_chains = 0;
        }
    } plan_scope{b->m};
    for (int i = 0; i < n; i++) b->m[i]->plan_chains = int(std::min<long long>(total, 1 << 30));
    for (int i = 0; i < n; i++) {
        nqes_ctx *c = b->m[i];
        const int rc = step_prepare(c, seeds[i], chains[i], samples[i], burn[i], lr[i], reglam[i], rtol[i], maxit[i],
                                    &arith[i]);
        if (rc) {  // this member's error; the others stay NQES_ERR_STATE (not run)
            if (statuses) statuses[i] = rc;
            b->err = "member " + std::to_string(i) + ": " + c->err;
            return rc;
        }
        tks[i] = choose_tk(c, chains[i]);
        // everything the captured nodes bake in: counts, arithmetic, launch shape,
        // precision, local-energy form, the options that select kernels, the
        // planned chains and the generation of the step buffers
        long long delta_bits = 0;
        std::memcpy(&delta_bits, &c->ham_delta, sizeof(delta_bits));
        keys[i] = {chains[i], samples[i], burn[i], arith[i], tks[i], c->step_precision, c->ham, delta_bits,
                   c->tensor_cores, c->reject_filter ? 1 : 0, c->mixed_exact_all ? 1 : 0, c->dw_force_warps,
                   c->dw_force_stage, (long long)c->buf_gen, total, c->stage_fault, c->mixed_e64};
    }
    // Capture (when the members changed), launch and wait. A failure here
    // means no member's step ran: each member's status becomes the error.
    auto capture_and_run = [&]() -> int {
    if (!b->exec || keys != b->keys) {
        NvtxRange r_build("batch graph capture");
        if (b->exec) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        b->keys.clear();
        // Graph: every member's sampling segment; ONE conditional while node
        // whose body holds every member's loop body (each guarded by its own
        // running flag) and then sets the loop condition from all the flags;
        // every member's update. The loop runs max over members of their
        // iteration counts, each member's kernels doing exactly the work of
        // its own loop and skipping once its solve has stopped.
        cudaGraph_t g = nullptr;
        if (cudaGraphCreate(&g, 0) != cudaSuccess) {
            b->err = "cudaGraphCreate failed";
            return NQES_ERR_CUDA;
        }
        auto fail = [&](int rc, const std::string &msg) {
            b->err = msg;
            cudaGraphDestroy(g);
            return rc;
        };
        std::vector<cudaGraphNode_t> nA(n);
        for (int i = 0; i < n; i++) {
            nqes_ctx *c = b->m[i];
            const int rc = arith[i] == NQES_ARITH_COMPLEX
                               ? add_member_sampling<cplx>(c, g, chains[i], samples[i], burn[i], tks[i], &nA[i])
                               : add_member_sampling<double>(c, g, chains[i], samples[i], burn[i], tks[i], &nA[i]);
            if (rc) return fail(rc, "member " + std::to_string(i) + ": " + c->err);
        }
        cudaGraphConditionalHandle cond;
        cudaError_t e = cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault);
        if (e != cudaSuccess) return fail(NQES_ERR_CUDA, std::string("cudaGraphConditionalHandleCreate: ") + cudaGetErrorString(e));
        cudaGraphNodeParams cp{};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = cond;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t nW;
        e = cudaGraphAddNode(&nW, g, nA.data(), nullptr, n, &cp);
        if (e != cudaSuccess) return fail(NQES_ERR_CUDA, std::string("cudaGraphAddNode (while): ") + cudaGetErrorString(e));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        BodyGroups grp;
        const int grc = plan_body_groups(b, arith, grp);
        if (grc) return fail(grc, b->err);
        e = cudaStreamBeginCaptureToGraph(b->st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return fail(NQES_ERR_CUDA, std::string("capture of the batched loop body: ") + cudaGetErrorString(e));
        cudaError_t le = capture_grouped_body(b, grp);
        if (le == cudaSuccess) le = launch_batch_cond(b->flags_d, n, cond, b->st);
        const cudaError_t ce = cudaStreamEndCapture(b->st, &body);
        if (le != cudaSuccess || ce != cudaSuccess)
            return fail(NQES_ERR_CUDA, std::string("capture of the batched loop body: ") +
                                           cudaGetErrorString(le != cudaSuccess ? le : ce));
        for (int i = 0; i < n; i++) {
            nqes_ctx *c = b->m[i];
            const int rc = arith[i] == NQES_ARITH_COMPLEX ? add_member_update<cplx>(c, g, nW)
                                                          : add_member_update<double>(c, g, nW);
            if (rc) return fail(rc, "member " + std::to_string(i) + ": " + c->err);
        }
        const cudaError_t ie = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            b->err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ie);
            return NQES_ERR_CUDA;
        }
        b->keys = keys;
    }
    for (int i = 0; i < n; i++) {
        nqes_ctx *c = b->m[i];
        if (cudaMemcpyAsync(c->sp, c->sp_host, sizeof(StepParams), cudaMemcpyHostToDevice, b->st) != cudaSuccess) {
            b->err = "step parameter copy failed";
            return NQES_ERR_CUDA;
        }
        c->last_tk = tks[i];
    }
    cudaEventRecord(b->ev0, b->st);
    cudaError_t le = cudaGraphLaunch(b->exec, b->st);
    cudaEventRecord(b->ev1, b->st);
    for (int i = 0; i < n && le == cudaSuccess; i++)
        if (step_readback(b->m[i], b->st)) le = cudaErrorUnknown;
    if (le == cudaSuccess) le = cudaStreamSynchronize(b->st);
    if (le != cudaSuccess) {
        b->err = std::string("batched step: ") + cudaGetErrorString(le);
        return NQES_ERR_CUDA;
    }
    return NQES_OK;
    };
    const int rc_run = capture_and_run();
    if (rc_run) {
        if (statuses)
            for (int i = 0; i < n; i++) statuses[i] = rc_run;
        return rc_run;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    if (ms_total) *ms_total = ms;
    int first = NQES_OK;
    for (int i = 0; i < n; i++) {
        const int rc = step_finish(b->m[i], chains[i], samples[i], burn[i], arith[i], maxit[i], ms,
                                   e_mats ? e_mats[i] : nullptr, infos ? &infos[i] : nullptr);
        if (statuses) statuses[i] = rc;
        if (rc && !first) {
            first = rc;
            b->err = "member " + std::to_string(i) + ": " + b->m[i]->err;
        }
    }
    return first;
}

}  // extern "C"
