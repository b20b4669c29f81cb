// Serving loop: continuous batching of SR solves on one GPU.
//
// No counterpart in the reference (one solve per process). Built only on the
// public C ABI (contexts and batches), so a solve's numbers are those of
// stepping it alone. A worker thread repeats:
//   admit   queued requests, oldest first, while the solve's device footprint
//           (nqes_footprint_bytes) fits the budget and an active slot is free;
//   step    every active solve once, as one batched launch (nqes_batch), with
//           the reference's schedules: lr = max(lr0 lr_decay^t, lr_cutoff),
//           reglam likewise, seed + t*chains (code/rbm.cc:1173-1183);
//   test    the reference's convergence rule (code/rbm.cc:1185-1194): sorted
//           real eigenvalues of e_mat/N, converged at step t > 0 when
//           |evals - best| < tol, best = the lowest-sum evals so far;
//   retire  converged solves, solves at max_steps and failed ones, freeing
//           their device memory and slot; results wait for nqes_server_poll.
//           A step that goes non-finite restarts the solve's run from its
//           initial weights with a new seed, up to 16 runs, as code/run.sh
//           does with the reference's exit code 127.
// Requests that arrive while others run join the next step's batch as memory
// and slots free up, so their work overlaps on the device.
//
// Solves of very different sizes would make one batch wait for its largest
// member every step (a step of N = 96, K = 4 takes ~100x one of N = 16), so
// the server runs kLanes such workers, one per size class (parameters P =
// K (N + M + N M) up to 5000, up to 20000, above), each with its own batch on
// its own stream: the lanes' steps run side by side on the GPU, and a small
// solve is never held back by a large one. The lanes share the queue (each
// takes the oldest request of its class), the device-memory budget, the slot
// count and the results.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/nqes.h"
#include "../cli/small_eig.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Solve {
    uint64_t id = 0;
    nqes_request r{};
    std::vector<double> J, a, b, w;
    Clock::time_point t_submit, t_admit;
    nqes_ctx *ctx = nullptr;
    uint64_t bytes = 0;
    int step = 0;
    int restarts = 0;     // restarts after a non-finite step (code/run.sh)
    uint64_t seed = 0;    // the current run's seed: the request's, moved on at each restart
    double lr = 0, reglam = 0;
    std::vector<double> evals, best;
    std::vector<std::complex<double>> emat;
};

constexpr int kLanes = 3;
constexpr int kMaxTries = 16;  // runs per solve, as code/run.sh's MAX_TRIES

// Size class of a request: its lane.
int lane_of(const nqes_request &r) {
    const long long P = (long long)r.n_states * (r.n_spins + r.n_hidden + (long long)r.n_spins * r.n_hidden);
    return P <= 5000 ? 0 : P <= 20000 ? 1 : 2;
}

// One lane: its worker's active solves and batch.
struct Lane {
    int index = 0;
    std::vector<Solve *> active;
    nqes_batch *batch = nullptr;
    // the batch's members by solve id: a retired solve's context is freed and a
    // new context may reuse its address, so pointers cannot tell batches apart
    std::vector<uint64_t> batch_members;
    int n_active = 0;  // published under the server's mutex
    std::thread worker;
};

}  // namespace

struct nqes_server {
    int device = 0;
    uint64_t budget = 0, in_use = 0;
    int max_active = 0;
    std::mutex mu;
    std::condition_variable cv;
    std::deque<Solve *> queue;
    std::deque<nqes_result> done;
    uint64_t next_id = 1;
    int slots_used = 0;  // admitted and not yet retired, all lanes (under mu)
    // cumulative worker time (seconds) by phase over the lanes, and counts, under mu
    double t_admit = 0, t_rebuild = 0, t_step = 0, t_post = 0;
    uint64_t n_steps = 0, n_rebuilds = 0;
    bool stop = false;
    Lane lanes[kLanes];
    std::string err;
};

namespace {

nqes_result make_result(const Solve &s, int status, int converged) {
    nqes_result res{};
    res.id = s.id;
    res.status = status;
    res.converged = converged;
    res.steps = s.step;
    res.n_states = s.r.n_states;
    for (int k = 0; k < s.r.n_states && k < 4; k++) {
        res.energies[k] = k < int(s.evals.size()) ? s.evals[k] : 0.0;
        res.best[k] = k < int(s.best.size()) ? s.best[k] : 0.0;
    }
    const auto now = Clock::now();
    res.t_queued = std::chrono::duration<double>(s.t_admit - s.t_submit).count();
    res.t_total = std::chrono::duration<double>(now - s.t_submit).count();
    res.footprint = s.bytes;
    res.restarts = s.restarts;
    return res;
}

// (Re)starts the solve's run from its initial weights with its current seed:
// the request's weights, else the reference initialisation from that seed.
int begin_run(Solve *s) {
    const nqes_request &r = s->r;
    const int st = !s->a.empty() ? nqes_set_weights(s->ctx, s->a.data(), s->b.data(), s->w.data())
                                 : nqes_init_weights(s->ctx, s->seed);
    s->step = 0;
    s->lr = r.lr0;
    s->reglam = r.reglam0;
    s->evals.clear();
    s->best.clear();
    return st;
}

// Creates the solve's context (worker thread). Returns the status.
int start_solve(nqes_server *srv, Solve *s) {
    const nqes_request &r = s->r;
    int st = nqes_create(r.n_spins, r.n_hidden, r.n_states, s->J.data(), r.h, srv->device, &s->ctx);
    if (st) return st;
    s->seed = r.seed;
    st = begin_run(s);
    if (!st) st = nqes_set_option(s->ctx, NQES_OPT_PRECISION, r.precision);
    s->emat.assign(size_t(r.n_states) * r.n_states, 0.0);
    return st;
}

void finish_solve(nqes_server *srv, Solve *s, int status, int converged) {
    nqes_result res = make_result(*s, status, converged);
    if (s->ctx) nqes_destroy(s->ctx);
    s->ctx = nullptr;
    std::lock_guard<std::mutex> g(srv->mu);
    srv->in_use -= s->bytes;
    srv->slots_used--;
    srv->done.push_back(res);
    delete s;
}

void worker_loop(nqes_server *srv, Lane *lane) {
    for (;;) {
        std::vector<Solve *> admitted;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            if (srv->stop) break;
            // the oldest queued requests of this lane's class, while memory and slots allow
            for (auto it = srv->queue.begin(); it != srv->queue.end() && srv->slots_used < srv->max_active;) {
                Solve *s = *it;
                if (lane_of(s->r) != lane->index) {
                    ++it;
                    continue;
                }
                if (srv->in_use + s->bytes > srv->budget) {
                    if (srv->slots_used == 0 && s->bytes > srv->budget) {
                        it = srv->queue.erase(it);  // can never fit: fail it
                        nqes_result res = make_result(*s, NQES_ERR_OOM, 0);
                        srv->done.push_back(res);
                        delete s;
                        continue;
                    }
                    break;  // oldest first: wait for memory
                }
                it = srv->queue.erase(it);
                srv->in_use += s->bytes;
                srv->slots_used++;
                admitted.push_back(s);
            }
            if (lane->active.empty() && admitted.empty()) {
                srv->cv.wait_for(lk, std::chrono::milliseconds(20));
                continue;
            }
        }
        const auto c0 = Clock::now();
        for (Solve *s : admitted) {
            s->t_admit = Clock::now();
            const int st = start_solve(srv, s);
            if (st)
                finish_solve(srv, s, st, 0);
            else
                lane->active.push_back(s);
        }
        if (lane->active.empty()) continue;

        // one batched step over the active solves
        const auto c1 = Clock::now();
        std::vector<nqes_ctx *> members;
        std::vector<uint64_t> ids;
        for (Solve *s : lane->active) {
            members.push_back(s->ctx);
            ids.push_back(s->id);
        }
        bool rebuilt = false;
        if (!lane->batch || ids != lane->batch_members) {
            rebuilt = true;
            if (lane->batch) nqes_batch_destroy(lane->batch);
            lane->batch = nullptr;
            if (nqes_batch_create(members.data(), int(members.size()), &lane->batch)) {
                for (Solve *s : lane->active) finish_solve(srv, s, NQES_ERR_CUDA, 0);
                lane->active.clear();
                continue;
            }
            lane->batch_members = ids;
        }
        const size_t n = lane->active.size();
        std::vector<uint64_t> seeds(n), maxit(n);
        std::vector<int> chains(n), m(n), burn(n), status(n);
        std::vector<double> lr(n), reglam(n), rtol(n);
        std::vector<double *> emats(n);
        for (size_t i = 0; i < n; i++) {
            const Solve *s = lane->active[i];
            const nqes_request &r = s->r;
            seeds[i] = s->seed + uint64_t(s->step) * r.chains;
            chains[i] = r.chains;
            m[i] = r.samples_per_chain;
            burn[i] = r.burn_in;
            lr[i] = std::max(s->lr, r.lr_cutoff);
            reglam[i] = std::max(s->reglam, r.reglam_cutoff);
            rtol[i] = r.minres_rtol;
            maxit[i] = r.minres_maxit;
            emats[i] = reinterpret_cast<double *>(lane->active[i]->emat.data());
        }
        const auto c2 = Clock::now();
        const int step_rc = nqes_batch_sr_step(lane->batch, seeds.data(), chains.data(), m.data(), burn.data(),
                                               lr.data(), reglam.data(), rtol.data(), maxit.data(), emats.data(),
                                               nullptr, status.data(), nullptr);
        if (step_rc != NQES_OK && step_rc != NQES_ERR_NONFINITE) {
            // kept for nqes_server_last_error: the failed members carry the status
            std::lock_guard<std::mutex> g(srv->mu);
            srv->err = "lane " + std::to_string(lane->index) + ": " + nqes_batch_last_error(lane->batch);
        }
        const auto c3 = Clock::now();
        std::vector<Solve *> keep;
        for (size_t i = 0; i < n; i++) {
            Solve *s = lane->active[i];
            const int K = s->r.n_states, N = s->r.n_spins;
            if (status[i] == NQES_ERR_STATE) {  // not run: another member failed first
                keep.push_back(s);
                continue;
            }
            if (status[i] == NQES_ERR_NONFINITE && s->restarts + 1 < kMaxTries) {
                // as code/run.sh does after a floating-point error: the run
                // again from the start with a new seed
                s->restarts++;
                s->seed = s->r.seed + (uint64_t(s->restarts) << 40);
                if (begin_run(s) == NQES_OK) {
                    keep.push_back(s);
                    continue;
                }
            }
            if (status[i]) {
                finish_solve(srv, s, status[i], 0);
                continue;
            }
            std::vector<std::complex<double>> A(s->emat), ev(K), vec(size_t(K) * K);
            for (auto &x : A) x /= double(N);
            nqes_cli::small_eig(A.data(), K, ev.data(), vec.data());
            s->evals.assign(K, 0.0);
            for (int k = 0; k < K; k++) s->evals[k] = ev[k].real();
            std::sort(s->evals.begin(), s->evals.end());
            s->lr *= s->r.lr_decay;
            s->reglam *= s->r.reglam_decay;
            double d2 = 0, s_new = 0, s_best = 0;
            if (s->step > 0)
                for (int k = 0; k < K; k++) {
                    d2 += (s->evals[k] - s->best[k]) * (s->evals[k] - s->best[k]);
                    s_new += s->evals[k];
                    s_best += s->best[k];
                }
            const bool conv = s->step > 0 && std::sqrt(d2) < s->r.tol;
            if (s->step == 0 || s_new < s_best) s->best = s->evals;
            s->step++;
            if (conv || s->step >= s->r.max_steps)
                finish_solve(srv, s, NQES_OK, conv ? 1 : 0);
            else
                keep.push_back(s);
        }
        lane->active.swap(keep);
        const auto c4 = Clock::now();
        auto sec = [](Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); };
        std::lock_guard<std::mutex> g(srv->mu);
        lane->n_active = int(lane->active.size());
        srv->t_admit += sec(c0, c1);
        srv->t_step += sec(c2, c3);
        srv->t_post += sec(c3, c4);
        srv->n_steps++;
        if (rebuilt) {
            srv->t_rebuild += sec(c1, c2);  // batch creation; its graph is captured inside the first step
            srv->n_rebuilds++;
        }
    }
    if (lane->batch) nqes_batch_destroy(lane->batch);
    lane->batch = nullptr;
    for (Solve *s : lane->active) {
        if (s->ctx) nqes_destroy(s->ctx);
        delete s;
    }
    lane->active.clear();
}

thread_local std::string g_server_error;

}  // namespace

extern "C" {

const char *nqes_server_last_error(const nqes_server *s) {
    if (!s) return g_server_error.c_str();
    thread_local std::string copy;  // the workers may set err meanwhile
    std::lock_guard<std::mutex> g(const_cast<nqes_server *>(s)->mu);
    copy = s->err;
    return copy.c_str();
}

int nqes_server_create(int device, uint64_t hbm_budget_bytes, int max_active, nqes_server **out) {
    if (!out || max_active < 1 || hbm_budget_bytes == 0) {
        g_server_error = "out must be non-NULL, max_active >= 1 and the budget positive";
        return NQES_ERR_INVALID;
    }
    nqes_server *s = new nqes_server();
    s->device = device;
    s->budget = hbm_budget_bytes;
    s->max_active = max_active;
    for (int l = 0; l < kLanes; l++) {
        s->lanes[l].index = l;
        s->lanes[l].worker = std::thread(worker_loop, s, &s->lanes[l]);
    }
    *out = s;
    return NQES_OK;
}

int nqes_server_submit(nqes_server *s, const nqes_request *r, uint64_t *id) {
    if (!s || !r || !r->J) return NQES_ERR_INVALID;
    if (r->n_states < 1 || r->n_states > 4 || r->n_spins < 1 || r->n_spins > 128 || r->n_hidden < 1 ||
        r->n_hidden > 512 || r->chains < 1 || r->samples_per_chain < 1 || r->burn_in < 0 || r->max_steps < 1 ||
        (r->precision != NQES_PRECISION_FP64 && r->precision != NQES_PRECISION_MIXED &&
         r->precision != NQES_PRECISION_CERTIFIED) || ((r->a == nullptr) != (r->b == nullptr)) ||
        ((r->a == nullptr) != (r->w == nullptr))) {
        std::lock_guard<std::mutex> g(s->mu);
        s->err = "invalid request";
        return NQES_ERR_INVALID;
    }
    Solve *v = new Solve();
    v->r = *r;
    const size_t N = r->n_spins, M = r->n_hidden, K = r->n_states;
    v->J.assign(r->J, r->J + N * N);
    bool cplx_w = false;
    if (r->a) {
        v->a.assign(r->a, r->a + 2 * K * N);
        v->b.assign(r->b, r->b + 2 * K * M);
        v->w.assign(r->w, r->w + 2 * K * N * M);
        for (size_t t = 1; t < v->w.size(); t += 2) cplx_w = cplx_w || v->w[t] != 0.0;
        for (size_t t = 1; t < v->a.size(); t += 2) cplx_w = cplx_w || v->a[t] != 0.0;
        for (size_t t = 1; t < v->b.size(); t += 2) cplx_w = cplx_w || v->b[t] != 0.0;
    } else {
        cplx_w = true;  // the reference's initialisation draws complex weights
    }
    v->r.J = nullptr;
    v->r.a = v->r.b = v->r.w = nullptr;
    nqes_footprint_bytes(r->n_spins, r->n_hidden, r->n_states, r->chains, r->samples_per_chain, r->precision,
                         cplx_w ? 1 : 0, &v->bytes);
    v->t_submit = Clock::now();
    uint64_t vid;
    {
        std::lock_guard<std::mutex> g(s->mu);
        vid = v->id = s->next_id++;
        s->queue.push_back(v);  // from here on a worker may admit, fail and free v
    }
    s->cv.notify_all();
    if (id) *id = vid;
    return NQES_OK;
}

int nqes_server_poll(nqes_server *s, nqes_result *out, int max_results, int *count) {
    if (!s || !count || (max_results > 0 && !out)) return NQES_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    int c = 0;
    while (c < max_results && !s->done.empty()) {
        out[c++] = s->done.front();
        s->done.pop_front();
    }
    *count = c;
    return NQES_OK;
}

int nqes_server_status(nqes_server *s, int *queued, int *active, int *done, uint64_t *bytes_in_use) {
    if (!s) return NQES_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    if (queued) *queued = int(s->queue.size());
    if (active) {
        *active = 0;
        for (const Lane &l : s->lanes) *active += l.n_active;
    }
    if (done) *done = int(s->done.size());
    if (bytes_in_use) *bytes_in_use = s->in_use;
    return NQES_OK;
}

int nqes_server_times(nqes_server *s, double *admit_s, double *rebuild_s, double *step_s, double *post_s,
                      uint64_t *steps, uint64_t *rebuilds) {
    if (!s) return NQES_ERR_INVALID;
    std::lock_guard<std::mutex> g(s->mu);
    if (admit_s) *admit_s = s->t_admit;
    if (rebuild_s) *rebuild_s = s->t_rebuild;
    if (step_s) *step_s = s->t_step;
    if (post_s) *post_s = s->t_post;
    if (steps) *steps = s->n_steps;
    if (rebuilds) *rebuilds = s->n_rebuilds;
    return NQES_OK;
}

int nqes_server_destroy(nqes_server *s) {
    if (!s) return NQES_OK;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    for (Lane &l : s->lanes)
        if (l.worker.joinable()) l.worker.join();
    for (Solve *v : s->queue) delete v;
    delete s;
    return NQES_OK;
}

}  // extern "C"
