/*
 * nqes.h — C ABI of the GB300 (sm_103a) VMC / stochastic-reconfiguration
 * library for K multi-RBM excited states (libnqes.so).
 *
 * The reference (cl91/nqes-trapped-ion) has no plugin or FFI: its hot path is
 * the function seam inside code/rbm.cc that its executable drives. Each entry
 * point below replaces one such seam; the comment names it (file:line).
 *
 * Conventions
 *   - Every call returns int status: NQES_OK (0) or a negative NQES_ERR_*;
 *     nqes_last_error(ctx) then describes the failure. No C++ exception
 *     crosses this boundary.
 *   - Complex arrays are interleaved (re, im) doubles (C99 double _Complex /
 *     std::complex<double> layout).
 *   - Weights use the reference layout (code/rbm.cc:121-132):
 *       a: K×N, b: K×M, w: K×N×M with w[(k*N+i)*M+j], all row-major.
 *   - A spin configuration is ceil(N/64) uint64 words, bit i set = spin i
 *     down (sigma_i = -1), as std::bitset in code/rbm.cc:77-83.
 *   - Parameter vectors (log-derivatives, forces, solutions) have length
 *     P = K*(N+M+N*M) in the layout [k][a_i | b_j | w_{i*M+j}]
 *     (code/rbm.cc:199-239).
 *   - The caller owns every host buffer; the context owns device memory.
 *     One host thread per context; a context is bound to one device and one
 *     CUDA stream. All results are computed on the GPU; there is no CPU path.
 */
#ifndef NQES_H
#define NQES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NQES_OK 0
#define NQES_ERR_CUDA (-1)       /* CUDA runtime error, or no CUDA device */
#define NQES_ERR_OOM (-2)        /* device allocation failed */
#define NQES_ERR_NONFINITE (-3)  /* non-finite amplitude ratio, energy, derivative or solver scalar */
#define NQES_ERR_TIMEOUT (-4)    /* a bounded device-side wait ran out */
#define NQES_ERR_INVALID (-5)    /* invalid argument or shape */
#define NQES_ERR_STATE (-6)      /* call out of order (e.g. no sampled step yet) */

/* Arithmetic of the device path (nqes_set_option NQES_OPT_ARITH). */
#define NQES_ARITH_AUTO 0     /* real if every weight has zero imaginary part, else complex */
#define NQES_ARITH_COMPLEX 1  /* always complex (the reference's own arithmetic) */
#define NQES_ARITH_REAL 2     /* real; rejected when a weight has a non-zero imaginary part */

/* Options (nqes_set_option). */
#define NQES_OPT_ARITH 1             /* NQES_ARITH_* (default AUTO) */
#define NQES_OPT_THREADS_PER_BLOCK 2 /* sampler threads per RBM column block: 32, 64, 128 or 0 = autotune */
#define NQES_OPT_MINRES_CAP 3        /* device-side MINRES-QLP iteration cap (default 100000) */
#define NQES_OPT_PRECISION 4         /* NQES_PRECISION_* (default FP64) */
#define NQES_OPT_REJECT_FILTER 5     /* 1: FP32 rejection filter in the FP64 real sampler; 0 (default): off.
                                      * The filter skips the FP64 work of proposals that a rigorous
                                      * FP32 bound proves rejected, in sweeps that follow a sweep with
                                      * under 50% acceptance; results are bit-identical either way. */
#define NQES_OPT_AUTOTUNE 7          /* 1: time the sampler's admissible launch shapes on the first step of
                                      * each (chains, samples, burn-in, precision, arithmetic) and keep the
                                      * fastest; 0 (default): occupancy-based choice. Results do not depend
                                      * on the launch shape beyond FP64 rounding of the product trees. */
#define NQES_OPT_TENSOR_CORES 8      /* 1 (default): in the MIXED form, the rows pass of the factored S·v
                                      * runs on the tensor cores (tcgen05, B split into three BF16 terms,
                                      * FP32 accumulation) where the shape allows (N <= 143, M <= 255) and
                                      * pays off (N M >= 4096); 2: wherever the shape allows; 0: FP32
                                      * CUDA cores. All agree to FP32 rounding. */
#define NQES_OPT_FUSED_SV 9          /* 1: with real arithmetic in the FP64 and CERTIFIED forms, S·v reads
                                      * the stored O once per product (one persistent kernel: u = O v and
                                      * O^T u per staged group of rows, double-float arithmetic on the FP32
                                      * pipe, within 1e-13 of FP64 sums) where P is even and at most 8192;
                                      * 0: two FP64 passes; -1 (default): on in CERTIFIED, off in FP64. */
#define NQES_OPT_MIXED_ENERGY64 11   /* local energies of the MIXED form's decision-warp sampler (O stays
                                      * as its FP32 factors): the N single-flip ratios as double-float
                                      * products of the tables on the FP32 pipe, with tanh of the exact
                                      * theta from its FP32 value plus the first-order term of theta's
                                      * low part (2, default) or in FP64 (1); 0: FP32 ratio products. */
#define NQES_OPT_TEST_STAGE_WAIT 10  /* test hook for the bounded device-side waits: 1 = the decision-warp
                                      * sampler stages its tables and its wait is for bytes that no copy
                                      * delivers, with a short poll limit, so the step returns
                                      * NQES_ERR_TIMEOUT and the context stays usable; 0 (default): off.
                                      * Only for shapes with that sampler (MIXED / CERTIFIED, real). */
#define NQES_OPT_MIXED_EXACT 6       /* 1: MIXED takes every accept decision by its exact FP64 path
                                      * (verification of that path); 0 (default): only when the FP32
                                      * bound cannot decide. */
#define NQES_OPT_SAMPLER_PLAN 12     /* launch plan of the decision-warp sampler (MIXED, CERTIFIED real):
                                      * 0 (default): planned from the chains (and the autotuner when on);
                                      * else the warps per chain (1, 2, 4 or 8), plus 16 to stage the step's
                                      * tables in shared memory. Results do not depend on the plan. */

/* Precision of the SR step (nqes_set_option NQES_OPT_PRECISION).
 * FP64: every quantity in FP64, as the reference.
 * MIXED (real weights only): factors, ratio products and accept decisions
 *   in FP32 with a certified error bound and an exact FP64 decision whenever
 *   the bound cannot decide, so the Markov chains are the FP64 chains;
 *   theta, Phi, local energies (NQES_OPT_MIXED_ENERGY64), moments' sums,
 *   MINRES-QLP and the update in FP64;
 *   log-derivatives stored as their FP32 factors (tanh rows, Phi coefficients)
 *   and S·v and the moments computed from them in FP32. */
#define NQES_PRECISION_FP64 0
#define NQES_PRECISION_MIXED 1
/* FP64 results (E, O, moments, S·v, MINRES-QLP, update as NQES_PRECISION_FP64)
 * with the mixed form's sampler: accept decisions from certified FP32 bounds
 * with the exact FP64 fallback, so the same configurations; real weights and
 * shapes of the decision-warp sampler (otherwise the FP64 sampler runs). */
#define NQES_PRECISION_CERTIFIED 2

typedef struct nqes_ctx nqes_ctx;

/* Result of one SR step. */
typedef struct nqes_step_info {
    int minres_flag;             /* MINRES-QLP exit flag, code/minresqlp.h:14-54 */
    int arith;                   /* NQES_ARITH_REAL or NQES_ARITH_COMPLEX actually used */
    uint64_t minres_iters;       /* iterations as the reference counts them */
    uint64_t qlp_iters;
    double relres, anorm, acond, xnorm;
    uint64_t accepted;           /* accepted proposals, all chains, burn-in included */
    uint64_t proposals;          /* chains * (burn_in + m) * K * N */
    int warnings;                /* bit 1: device-side MINRES cap reached */
    double eloc_re, eloc_im;     /* mean local energy (trace of e_mat) */
    double ms_total;             /* device time of the step, CUDA events */
    uint64_t kernel_launches;    /* kernels this step launched (graph nodes run, loop bodies counted) */
    int precision;               /* NQES_PRECISION_* used */
    uint64_t exact_decisions;    /* MIXED: accept decisions the FP32 bound left to the exact FP64 path */
} nqes_step_info;

/* Kernels nqes_time_kernel can time in isolation. */
#define NQES_KERNEL_SAMPLE 1   /* the sampler: one CTA per chain, whole chains */
#define NQES_KERNEL_SV_ROWS 2  /* u = O v over the stored log-derivatives */
#define NQES_KERNEL_SV_COLS 3  /* y = O^H u over the stored log-derivatives */
#define NQES_KERNEL_MOMENTS 4  /* o, <|O|^2>, <E conj O> column reductions */
#define NQES_KERNEL_SV 5       /* the step's S·v passes (the fused kernel where NQES_OPT_FUSED_SV applies) */

/* Create a context for N spins, M hidden units, K states on CUDA `device`,
 * for H = sum_{i!=j} J_ij sz_i sz_j - h sum_i sx_i with the diagonal term
 * evaluated as 2 sum_{i>j} J[i*N+j] s_i s_j (lower triangle of the row-major
 * N×N J).  Replaces the compile-time shape, the compiled-in J (JMAT_INC) and
 * the `hamiltonian` callable of code/rbm.cc:1011-1062, 1273-1313.
 * Limits: 1 <= K <= 4, 1 <= N <= 128, 1 <= M <= 512. */
int nqes_create(int n_spins, int n_hidden, int n_states, const double *J, double h, int device, nqes_ctx **out);
int nqes_destroy(nqes_ctx *ctx);
/* Description of the last failure on ctx (or of the calling thread's last
 * failed nqes_create when ctx is NULL). Valid until the next call on the same
 * context (in the same thread). */
const char *nqes_last_error(const nqes_ctx *ctx);
int nqes_set_option(nqes_ctx *ctx, int option, int64_t value);

/* Local-energy form (nqes_set_hamiltonian). */
#define NQES_HAM_ISING_LIKE 0      /* the nqes_create form: ising, periodicising, longrange, trappedion
                                      (ising_like_hamiltonian, code/rbm.cc:1033-1062) */
#define NQES_HAM_HEISENBERG_LIKE 1 /* H = sum_{i>j} J_ij (sx_i sx_j + sy_i sy_j + delta sz_i sz_j) with the
                                      lower triangle of the nqes_create J: hs (J_ij = 1/d_ij^2, delta 1)
                                      and xxz (J = -1 on the periodic chain's bonds, delta -1)
                                      (hs_like_hamiltonian, code/rbm.cc:1064-1119); h is unused.
                                      FP64 form only (NQES_PRECISION_FP64). */
/* Select the local-energy form of the following SR steps, evaluations and
 * runs. Replaces the choice of the `hamiltonian` callable in code/rbm.cc:1293-1325. */
int nqes_set_hamiltonian(nqes_ctx *ctx, int form, double delta);

/* Weights, reference layout, complex interleaved.  Replaces the in-memory
 * MultiRBM of code/rbm.cc:127-132 (load_rbm / dump_rbm read and write it). */
int nqes_set_weights(nqes_ctx *ctx, const double *a, const double *b, const double *w);
int nqes_get_weights(nqes_ctx *ctx, double *a, double *b, double *w);
/* Reference initialisation: init_multi_rbm with pcg64(seed - 1) and
 * std::normal_distribution<double>, code/rbm.cc:241-270, 1127, 1146-1147. */
int nqes_init_weights(nqes_ctx *ctx, uint64_t seed);

/* One SR step: sample, local energies, log-derivatives, moments, matrix-free
 * MINRES-QLP solve of (S + reglam diag S) x = f, and w -= lr x.
 * Replaces monte_carlo(rbm, seed, ncpus, m, burn_in, lr, reglam, rtol, maxit,
 * hamiltonian), code/rbm.cc:564-719 (chain c uses pcg64(seed + c), so pass
 * seed + iter*chains as code/rbm.cc:1179 does).  e_mat receives the K×K
 * complex matrix the reference returns (e_mat / Ns, not yet divided by N). */
int nqes_sr_step(nqes_ctx *ctx, uint64_t seed, int chains, int samples_per_chain, int burn_in, double lr,
                 double reglam, double rtol, uint64_t maxit, double *e_mat, nqes_step_info *info);

/* Correlation functions x, z (N×K) and xx, zz (N*N×K), row-major
 * [row][state], unsorted: res(i,k) = Re diag(V^-1 <Phi^-1 F_i> V)_k for the
 * K×K eigenvector matrix V (evecs, row-major complex).  Replaces the four
 * correlation_fcn passes of code/rbm.cc:730-771, 1206-1217, which share one
 * seed and therefore one set of chains. */
int nqes_correlations(nqes_ctx *ctx, uint64_t seed, int chains, int samples_per_chain, int burn_in,
                      const double *evecs, double *x, double *z, double *xx, double *zz);

/* ---- inspection (parity tests and diagnostics) ---- */

/* Phi (K×K complex, row-major, unscaled), tanh(theta) (M×K² complex,
 * column k*K+kk), E = Phi^-1 H Phi (K×K complex) and O (P complex) at `count`
 * given configurations (count × K × ceil(N/64) words); any output may be
 * NULL.  The same device code the sampler runs per sample (state_fcn,
 * ising_like_hamiltonian or hs_like_hamiltonian, deriv: code/rbm.cc:146-171,
 * 1042-1062, 1091-1119, 199-239).  Where Phi is rank deficient (e.g. two equal
 * rows, as the --dump-* enumerations of code/rbm.cc:473-524 meet them), E uses
 * the Moore-Penrose pseudo-inverse, the reference's pseudoInverse(), and O is
 * zero. */
int nqes_evaluate(nqes_ctx *ctx, const uint64_t *configs, int count, double *phi, double *tanh_theta, double *E,
                  double *O);
/* Per-sample records of the last SR step: configurations (Ns × K × words),
 * local energies tr E (Ns complex) and E matrices (Ns × K² complex). */
int nqes_get_samples(nqes_ctx *ctx, uint64_t *configs, double *eloc, double *E);
/* Accepted proposals per chain (chains entries) of the last SR step. */
int nqes_get_accepts(nqes_ctx *ctx, uint64_t *accepted);
/* Rows [first, first+count) of the last step's O (count × P complex). */
int nqes_get_O(nqes_ctx *ctx, int first, int count, double *O);
/* Moments of the last step: o = <O>, skk = reglam(<|O|^2>-|o|^2), f (P complex each). */
int nqes_get_moments(nqes_ctx *ctx, double *o, double *skk, double *f);
/* Solution x of the last step's MINRES-QLP solve (P complex). */
int nqes_get_solution(nqes_ctx *ctx, double *x);
/* out = S v with the last step's samples and moments (P complex). */
int nqes_apply_S(nqes_ctx *ctx, const double *v, double *out);
/* Average device time (ms, CUDA events on the context's stream) of `reps`
 * back-to-back launches of one kernel (NQES_KERNEL_*) on the last step's
 * shapes and data, and the algorithmic bytes one launch moves (inputs read +
 * outputs written once). For benchmarks; re-running the sampler overwrites
 * the last step's samples (same seed, the current weights: after an SR step
 * these are the updated ones, so the samples change). */
int nqes_time_kernel(nqes_ctx *ctx, int kernel, int reps, double *avg_ms, double *algorithmic_bytes);

/* ---- S·v without allocation ----
 * No counterpart in the reference (its S·v is a lambda inside monte_carlo,
 * code/rbm.cc:660-683); this entry point exists for callers that cannot call
 * cudaMalloc: code running while a CUDA graph is being captured, hosts whose
 * device memory is owned by their own pool allocator, and loops that cannot
 * afford the synchronisation of cudaMalloc/cudaFree.
 * out = S v = (1/n_samples) O^H (O v) + skk∘v - (o·v) conj(o), where every
 * pointer is DEVICE memory the caller owns: O is n_samples × n_params
 * row-major, o, skk, v and out have n_params entries; complex_arith = 1 means
 * interleaved complex doubles, 0 means real doubles. `stream` is the
 * cudaStream_t to run on (NULL: the default stream of the current device);
 * the call runs on the stream's device, makes it current meanwhile, and
 * returns once the work is queued.
 * Intermediates live in a 16 MiB file-scope device array that every GPU
 * loading the library holds until exit; n_samples + n_params + ceil(n_params/256)
 * scalars must fit in it, larger sizes are rejected with NQES_ERR_INVALID.
 * The first call on a device looks the array's address up for that device
 * (make it before any stream capture). Calls share the array: overlapping
 * calls race.
 * Errors are described by nqes_last_error(NULL). */
int nqes_apply_S_static(const double *O, const double *o, const double *skk, const double *v, double *out,
                        int64_t n_samples, int64_t n_params, int complex_arith, void *stream);

/* Upper bound of the device memory (bytes) a context of this shape holds
 * while it runs SR steps of `chains` x `samples_per_chain` samples
 * (precision NQES_PRECISION_*, complex_arith 0/1). No GPU needed. */
int nqes_footprint_bytes(int n_spins, int n_hidden, int n_states, int chains, int samples_per_chain, int precision,
                         int complex_arith, uint64_t *bytes);

/* ---- batched multi-solve ----
 * No counterpart in the reference (it runs one solve per process). A batch
 * runs one SR step of every member context in ONE CUDA graph launch: each
 * member's step (sampling segment, MINRES-QLP while loop, update) is an
 * independent branch of the graph, so solves of different shapes overlap on
 * the GPU. Each member's results are exactly those of nqes_sr_step on it.
 * Members stay owned by the caller and must outlive the batch (a graph
 * captured for a member keeps its device buffers), live on one device, may differ in N, M,
 * K, J, h and precision, and may also be stepped on their own; the batch
 * re-captures its graph when a member's step shape changes. Errors are
 * described by nqes_batch_last_error (NULL: the last failed create). */
typedef struct nqes_batch nqes_batch;
int nqes_batch_create(nqes_ctx *const *members, int count, nqes_batch **out);
int nqes_batch_destroy(nqes_batch *batch);
const char *nqes_batch_last_error(const nqes_batch *batch);
/* One SR step of every member; every array has `count` entries in member
 * order, with nqes_sr_step's meaning. e_mats (or an entry) and infos may be
 * NULL; statuses (may be NULL) receives each member's status: NQES_ERR_STATE for
 * every other member when one member's arguments or buffers failed (none ran),
 * the error itself for every member when the capture, launch or wait failed;
 * ms_total (may be NULL) the device time of the batched launch. Returns the
 * first member error. */
int nqes_batch_sr_step(nqes_batch *batch, const uint64_t *seeds, const int *chains, const int *samples_per_chain,
                       const int *burn_in, const double *lr, const double *reglam, const double *rtol,
                       const uint64_t *maxit, double *const *e_mats, nqes_step_info *infos, int *statuses,
                       double *ms_total);

/* ---- serving loop ----
 * No counterpart in the reference. A server owns a worker thread on one GPU.
 * It admits submitted solves, oldest first, while the solve's device footprint
 * (nqes_footprint_bytes) fits the budget and an active slot is free; runs one
 * batched SR step over every admitted solve per iteration (nqes_batch) with
 * the reference's schedules (code/rbm.cc:1173-1183); applies the reference's
 * convergence test to each (sorted real eigenvalues of e_mat/N; converged at
 * step t > 0 when |evals - best| < tol, best = lowest-sum evals so far,
 * code/rbm.cc:1185-1194); restarts a solve whose step goes non-finite from
 * its initial weights with a new seed, up to 16 runs (code/run.sh); and
 * retires a solve when it converges, reaches max_steps or fails. Solves
 * submitted while others run join the next step. Three workers (lanes) by
 * size class, P up to 5000, up to 20000 and beyond, each batch their solves
 * side by side on the GPU. A solve's numbers equal those of running it alone. */
typedef struct nqes_server nqes_server;
typedef struct nqes_request {
    int n_spins, n_hidden, n_states;
    const double *J;                 /* N×N, copied at submit */
    double h;
    const double *a, *b, *w;         /* initial weights (copied), or all NULL: nqes_init_weights(seed) */
    uint64_t seed;                   /* step t uses seed + t*chains */
    int chains, samples_per_chain, burn_in;
    double lr0, lr_decay, lr_cutoff, reglam0, reglam_decay, reglam_cutoff;
    double minres_rtol;
    uint64_t minres_maxit;
    double tol;
    int max_steps;
    int precision;                   /* NQES_PRECISION_* */
} nqes_request;
typedef struct nqes_result {
    uint64_t id;
    int status;                      /* NQES_OK, NQES_ERR_OOM (never fits the budget) or a step's error */
    int converged;                   /* 1: tol met; 0: max_steps reached (or failed) */
    int steps;
    int n_states;
    double energies[4];              /* last step's sorted per-site energies */
    double best[4];                  /* lowest-sum energies seen */
    double t_queued, t_total;        /* seconds from submit to admission and to completion */
    uint64_t footprint;              /* device bytes reserved for the solve */
    int restarts;                    /* runs restarted after a non-finite step (new seed, as code/run.sh) */
} nqes_result;
int nqes_server_create(int device, uint64_t hbm_budget_bytes, int max_active, nqes_server **out);
/* Copies the request; returns at once with its id. Thread-safe. */
int nqes_server_submit(nqes_server *server, const nqes_request *request, uint64_t *id);
/* Moves up to max_results finished solves to out (oldest first). */
int nqes_server_poll(nqes_server *server, nqes_result *out, int max_results, int *count);
int nqes_server_status(nqes_server *server, int *queued, int *active, int *done, uint64_t *bytes_in_use);
/* Cumulative worker time by phase (seconds): admitting solves (context
 * creation, weights), creating batches after the active set changed, batched
 * SR steps (including the graph capture of a new batch), and the host-side
 * convergence tests and retirement; and the counts of steps and batch
 * rebuilds. Any output may be NULL. */
int nqes_server_times(nqes_server *server, double *admit_s, double *rebuild_s, double *step_s, double *post_s,
                      uint64_t *steps, uint64_t *rebuilds);
/* Stops the worker after its current step; unfinished solves are dropped. */
int nqes_server_destroy(nqes_server *server);
/* The last error: of a rejected submit, or of a batched step that failed
 * (its lane and the batch's message; the members carry the status). Valid in
 * the calling thread until its next call. NULL: the last failed create. */
const char *nqes_server_last_error(const nqes_server *server);

#ifdef __cplusplus
}
#endif
#endif /* NQES_H */
