"""Python host mirror of libnqes (include/nqes.h) over ctypes.

The reference drives its hot path through three functions of code/rbm.cc:
monte_carlo (one SR step, 564-719), correlation_fcn (730-771) and the weight
state (load_rbm / dump_rbm / init_multi_rbm). `Context` exposes the same
operations with the same argument meanings: `sr_step` takes the per-step seed
(seed + iter*chains, code/rbm.cc:1179), chains, samples per chain, burn-in,
learning rate, lambda, MINRES-QLP rtol and maxit, updates the weights in place
and returns the K×K matrix e_mat / Ns.

Everything runs in the CUDA library; this module only moves arrays. If the
library has not been built, `load_library` raises instead of falling back.
"""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libnqes.so")

OK = 0
ERR_CUDA, ERR_OOM, ERR_NONFINITE, ERR_TIMEOUT, ERR_INVALID, ERR_STATE = -1, -2, -3, -4, -5, -6
ARITH_AUTO, ARITH_COMPLEX, ARITH_REAL = 0, 1, 2
OPT_ARITH, OPT_THREADS_PER_BLOCK, OPT_MINRES_CAP, OPT_PRECISION = 1, 2, 3, 4
OPT_REJECT_FILTER, OPT_MIXED_EXACT, OPT_AUTOTUNE, OPT_TENSOR_CORES = 5, 6, 7, 8
OPT_FUSED_SV, OPT_TEST_STAGE_WAIT, OPT_MIXED_ENERGY64, OPT_SAMPLER_PLAN = 9, 10, 11, 12
PRECISION_FP64, PRECISION_MIXED, PRECISION_CERTIFIED = 0, 1, 2
HAM_ISING_LIKE, HAM_HEISENBERG_LIKE = 0, 1

EXPORTS = [
    "nqes_create", "nqes_destroy", "nqes_last_error", "nqes_set_option", "nqes_set_weights", "nqes_get_weights",
    "nqes_init_weights", "nqes_sr_step", "nqes_correlations", "nqes_evaluate", "nqes_get_samples",
    "nqes_get_accepts", "nqes_get_O", "nqes_get_moments", "nqes_get_solution", "nqes_apply_S", "nqes_time_kernel",
    "nqes_apply_S_static", "nqes_batch_create", "nqes_batch_destroy", "nqes_batch_last_error", "nqes_batch_sr_step",
    "nqes_footprint_bytes", "nqes_server_create", "nqes_server_submit", "nqes_server_poll", "nqes_server_status",
    "nqes_server_destroy", "nqes_server_last_error", "nqes_server_times", "nqes_set_hamiltonian",
]
KERNEL_SAMPLE, KERNEL_SV_ROWS, KERNEL_SV_COLS, KERNEL_MOMENTS, KERNEL_SV = 1, 2, 3, 4, 5


class NqesError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"libnqes error {status}: {message}")
        self.status = status


class StepInfo(ctypes.Structure):
    _fields_ = [
        ("minres_flag", ctypes.c_int), ("arith", ctypes.c_int),
        ("minres_iters", ctypes.c_uint64), ("qlp_iters", ctypes.c_uint64),
        ("relres", ctypes.c_double), ("anorm", ctypes.c_double), ("acond", ctypes.c_double),
        ("xnorm", ctypes.c_double), ("accepted", ctypes.c_uint64), ("proposals", ctypes.c_uint64),
        ("warnings", ctypes.c_int), ("eloc_re", ctypes.c_double), ("eloc_im", ctypes.c_double),
        ("ms_total", ctypes.c_double), ("kernel_launches", ctypes.c_uint64),
        ("precision", ctypes.c_int), ("exact_decisions", ctypes.c_uint64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_LIB = None


class Request(ctypes.Structure):
    """nqes_request (include/nqes.h)."""
    _fields_ = [("n_spins", ctypes.c_int), ("n_hidden", ctypes.c_int), ("n_states", ctypes.c_int),
                ("J", ctypes.POINTER(ctypes.c_double)), ("h", ctypes.c_double),
                ("a", ctypes.POINTER(ctypes.c_double)), ("b", ctypes.POINTER(ctypes.c_double)),
                ("w", ctypes.POINTER(ctypes.c_double)), ("seed", ctypes.c_uint64), ("chains", ctypes.c_int),
                ("samples_per_chain", ctypes.c_int), ("burn_in", ctypes.c_int), ("lr0", ctypes.c_double),
                ("lr_decay", ctypes.c_double), ("lr_cutoff", ctypes.c_double), ("reglam0", ctypes.c_double),
                ("reglam_decay", ctypes.c_double), ("reglam_cutoff", ctypes.c_double),
                ("minres_rtol", ctypes.c_double), ("minres_maxit", ctypes.c_uint64), ("tol", ctypes.c_double),
                ("max_steps", ctypes.c_int), ("precision", ctypes.c_int)]


class Result(ctypes.Structure):
    """nqes_result (include/nqes.h)."""
    _fields_ = [("id", ctypes.c_uint64), ("status", ctypes.c_int), ("converged", ctypes.c_int),
                ("steps", ctypes.c_int), ("n_states", ctypes.c_int), ("energies", ctypes.c_double * 4),
                ("best", ctypes.c_double * 4), ("t_queued", ctypes.c_double), ("t_total", ctypes.c_double),
                ("footprint", ctypes.c_uint64), ("restarts", ctypes.c_int)]

    def as_dict(self):
        k = self.n_states
        return {"id": self.id, "status": self.status, "converged": bool(self.converged), "steps": self.steps,
                "energies": list(self.energies[:k]), "best": list(self.best[:k]), "t_queued": self.t_queued,
                "t_total": self.t_total, "footprint": self.footprint, "restarts": self.restarts}
_dp = ctypes.POINTER(ctypes.c_double)
_u64p = ctypes.POINTER(ctypes.c_uint64)


def load_library(path=None):
    """Load libnqes.so; raises when it is missing (there is no CPU path)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(p)
    vp, i, d, u64, i64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64, ctypes.c_int64
    sigs = {
        "nqes_create": (i, [i, i, i, _dp, d, i, ctypes.POINTER(vp)]),
        "nqes_destroy": (i, [vp]),
        "nqes_last_error": (ctypes.c_char_p, [vp]),
        "nqes_set_option": (i, [vp, i, i64]),
        "nqes_set_hamiltonian": (i, [vp, i, d]),
        "nqes_set_weights": (i, [vp, _dp, _dp, _dp]),
        "nqes_get_weights": (i, [vp, _dp, _dp, _dp]),
        "nqes_init_weights": (i, [vp, u64]),
        "nqes_sr_step": (i, [vp, u64, i, i, i, d, d, d, u64, _dp, ctypes.POINTER(StepInfo)]),
        "nqes_correlations": (i, [vp, u64, i, i, i, _dp, _dp, _dp, _dp, _dp]),
        "nqes_evaluate": (i, [vp, _u64p, i, _dp, _dp, _dp, _dp]),
        "nqes_get_samples": (i, [vp, _u64p, _dp, _dp]),
        "nqes_get_accepts": (i, [vp, _u64p]),
        "nqes_get_O": (i, [vp, i, i, _dp]),
        "nqes_get_moments": (i, [vp, _dp, _dp, _dp]),
        "nqes_get_solution": (i, [vp, _dp]),
        "nqes_apply_S": (i, [vp, _dp, _dp]),
        "nqes_time_kernel": (i, [vp, i, i, _dp, _dp]),
        "nqes_apply_S_static": (i, [vp, vp, vp, vp, vp, i64, i64, i, vp]),
        "nqes_footprint_bytes": (i, [i, i, i, i, i, i, i, ctypes.POINTER(u64)]),
        "nqes_server_create": (i, [i, u64, i, ctypes.POINTER(vp)]),
        "nqes_server_submit": (i, [vp, ctypes.POINTER(Request), ctypes.POINTER(u64)]),
        "nqes_server_poll": (i, [vp, ctypes.POINTER(Result), i, ctypes.POINTER(i)]),
        "nqes_server_status": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(u64)]),
        "nqes_server_destroy": (i, [vp]),
        "nqes_server_times": (i, [vp, _dp, _dp, _dp, _dp, ctypes.POINTER(u64), ctypes.POINTER(u64)]),
        "nqes_server_last_error": (ctypes.c_char_p, [vp]),
        "nqes_batch_create": (i, [ctypes.POINTER(vp), i, ctypes.POINTER(vp)]),
        "nqes_batch_destroy": (i, [vp]),
        "nqes_batch_last_error": (ctypes.c_char_p, [vp]),
        "nqes_batch_sr_step": (i, [vp, _u64p, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i), _dp, _dp, _dp,
                                   _u64p, ctypes.POINTER(_dp), ctypes.POINTER(StepInfo), ctypes.POINTER(i), _dp]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def _cp(a):
    """complex128 array -> pointer to its interleaved doubles (None passes NULL)."""
    if a is None:
        return None
    return a.view(np.float64).ctypes.data_as(_dp)


def synthetic_j(n, alpha=1.2):
    """Power-law chain coupling J_ij = |i-j|^-alpha (i != j), zero diagonal, max |J| = 1."""
    i = np.arange(n)
    d = np.abs(i[:, None] - i[None, :]).astype(float)
    with np.errstate(divide="ignore"):
        J = np.where(d > 0, d ** (-alpha), 0.0)
    return J / np.max(np.abs(J)) if n > 1 else J


def synthetic_weights(n, m, k, sigma=0.01, seed=0, real=True):
    """Seeded N(0, sigma^2) weights in the reference layout (complex128, zero imaginary part when real)."""
    rng = np.random.default_rng(seed)

    def draw(shape):
        z = rng.normal(0.0, sigma, size=shape)
        if not real:
            z = z + 1j * rng.normal(0.0, sigma, size=shape)
        return np.ascontiguousarray(z, dtype=np.complex128)

    return draw((k, n)), draw((k, m)), draw((k, n, m))


class Context:
    """One solve (N spins, M hidden units, K states) resident on one GPU."""

    def __init__(self, n_spins, n_hidden, n_states, J, h, device=0, lib=None):
        self.lib = lib or load_library()
        self.N, self.M, self.K = int(n_spins), int(n_hidden), int(n_states)
        self.L = self.N + self.M + self.N * self.M
        self.P = self.K * self.L
        self.NW = (self.N + 63) // 64
        Jc = np.ascontiguousarray(J, dtype=np.float64)
        if Jc.shape != (self.N, self.N):
            raise ValueError("J must be N x N")
        h_ = ctypes.c_void_p()
        st = self.lib.nqes_create(self.N, self.M, self.K, Jc.ctypes.data_as(_dp), float(h), int(device),
                                  ctypes.byref(h_))
        if st != OK:
            raise NqesError(st, self.lib.nqes_last_error(None).decode())
        self._h = h_
        self.chains = 0

    def _check(self, st):
        if st != OK:
            raise NqesError(st, self.lib.nqes_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self.lib.nqes_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_option(self, option, value):
        self._check(self.lib.nqes_set_option(self._h, option, int(value)))

    def set_hamiltonian(self, form, delta=0.0):
        """HAM_ISING_LIKE (the create-time J and h) or HAM_HEISENBERG_LIKE
        (J_ij (sx sx + sy sy + delta sz sz) over the same J)."""
        self._check(self.lib.nqes_set_hamiltonian(self._h, int(form), float(delta)))

    def set_weights(self, a, b, w):
        a = np.ascontiguousarray(a, np.complex128).reshape(self.K, self.N)
        b = np.ascontiguousarray(b, np.complex128).reshape(self.K, self.M)
        w = np.ascontiguousarray(w, np.complex128).reshape(self.K, self.N, self.M)
        self._check(self.lib.nqes_set_weights(self._h, _cp(a), _cp(b), _cp(w)))

    def get_weights(self):
        a = np.zeros((self.K, self.N), np.complex128)
        b = np.zeros((self.K, self.M), np.complex128)
        w = np.zeros((self.K, self.N, self.M), np.complex128)
        self._check(self.lib.nqes_get_weights(self._h, _cp(a), _cp(b), _cp(w)))
        return a, b, w

    def init_weights(self, seed):
        self._check(self.lib.nqes_init_weights(self._h, int(seed)))

    def sr_step(self, seed, chains, samples_per_chain, burn_in, lr, reglam, rtol, maxit):
        emat = np.zeros((self.K, self.K), np.complex128)
        info = StepInfo()
        self._check(self.lib.nqes_sr_step(self._h, int(seed), int(chains), int(samples_per_chain), int(burn_in),
                                          float(lr), float(reglam), float(rtol), int(maxit), _cp(emat),
                                          ctypes.byref(info)))
        self.chains = int(chains)
        self.ns = int(chains) * int(samples_per_chain)
        return emat, info.as_dict()

    def correlations(self, seed, chains, samples_per_chain, burn_in, evecs):
        N, K = self.N, self.K
        ev = np.ascontiguousarray(evecs, np.complex128)
        x = np.zeros((N, K))
        z = np.zeros((N, K))
        xx = np.zeros((N * N, K))
        zz = np.zeros((N * N, K))
        p = lambda arr: arr.ctypes.data_as(_dp)
        self._check(self.lib.nqes_correlations(self._h, int(seed), int(chains), int(samples_per_chain),
                                               int(burn_in), _cp(ev), p(x), p(z), p(xx), p(zz)))
        return x, z, xx, zz

    def evaluate(self, configs):
        cfg = np.ascontiguousarray(configs, np.uint64).reshape(-1, self.K, self.NW)
        n = cfg.shape[0]
        K, M = self.K, self.M
        phi = np.zeros((n, K, K), np.complex128)
        th = np.zeros((n, M, K * K), np.complex128)
        E = np.zeros((n, K, K), np.complex128)
        O = np.zeros((n, self.P), np.complex128)
        self._check(self.lib.nqes_evaluate(self._h, cfg.ctypes.data_as(_u64p), n, _cp(phi), _cp(th), _cp(E),
                                           _cp(O)))
        return phi, th, E, O

    def get_samples(self):
        spins = np.zeros((self.ns, self.K, self.NW), np.uint64)
        eloc = np.zeros(self.ns, np.complex128)
        E = np.zeros((self.ns, self.K, self.K), np.complex128)
        self._check(self.lib.nqes_get_samples(self._h, spins.ctypes.data_as(_u64p), _cp(eloc), _cp(E)))
        return spins, eloc, E

    def get_accepts(self):
        acc = np.zeros(self.chains, np.uint64)
        self._check(self.lib.nqes_get_accepts(self._h, acc.ctypes.data_as(_u64p)))
        return acc

    def get_O(self, first, count):
        O = np.zeros((count, self.P), np.complex128)
        self._check(self.lib.nqes_get_O(self._h, int(first), int(count), _cp(O)))
        return O

    def get_moments(self):
        o = np.zeros(self.P, np.complex128)
        s = np.zeros(self.P, np.complex128)
        f = np.zeros(self.P, np.complex128)
        self._check(self.lib.nqes_get_moments(self._h, _cp(o), _cp(s), _cp(f)))
        return o, s, f

    def get_solution(self):
        x = np.zeros(self.P, np.complex128)
        self._check(self.lib.nqes_get_solution(self._h, _cp(x)))
        return x

    def time_kernel(self, kernel, reps=5):
        """(average ms, algorithmic bytes per launch) of one kernel on the last step's data."""
        ms = ctypes.c_double()
        by = ctypes.c_double()
        self._check(self.lib.nqes_time_kernel(self._h, int(kernel), int(reps), ctypes.byref(ms), ctypes.byref(by)))
        return ms.value, by.value

    def apply_S(self, v):
        v = np.ascontiguousarray(v, np.complex128)
        out = np.zeros(self.P, np.complex128)
        self._check(self.lib.nqes_apply_S(self._h, _cp(v), _cp(out)))
        return out


class Batch:
    """One SR step of several contexts (any shapes, same device) per CUDA graph launch."""

    def __init__(self, contexts, lib=None):
        self.lib = lib or load_library()
        self.members = list(contexts)
        arr = (ctypes.c_void_p * len(self.members))(*[c._h for c in self.members])
        h_ = ctypes.c_void_p()
        st = self.lib.nqes_batch_create(arr, len(self.members), ctypes.byref(h_))
        if st != OK:
            raise NqesError(st, self.lib.nqes_batch_last_error(None).decode())
        self._h = h_

    def close(self):
        if getattr(self, "_h", None):
            self.lib.nqes_batch_destroy(self._h)
            self._h = None

    def sr_step(self, seeds, chains, samples_per_chain, burn_in, lr, reglam, rtol, maxit):
        """Per-member arguments (sequences, member order); returns (e_mats, infos, statuses, ms_total)."""
        n = len(self.members)
        ci = ctypes.c_int * n
        cd = ctypes.c_double * n
        cu = ctypes.c_uint64 * n
        emats = [np.zeros((c.K, c.K), np.complex128) for c in self.members]
        eptr = (_dp * n)(*[_cp(e) for e in emats])
        infos = (StepInfo * n)()
        stat = ci()
        ms = ctypes.c_double()
        st = self.lib.nqes_batch_sr_step(self._h, cu(*map(int, seeds)), ci(*map(int, chains)),
                                         ci(*map(int, samples_per_chain)), ci(*map(int, burn_in)), cd(*map(float, lr)),
                                         cd(*map(float, reglam)), cd(*map(float, rtol)), cu(*map(int, maxit)), eptr,
                                         infos, stat, ctypes.byref(ms))
        if st != OK:
            raise NqesError(st, self.lib.nqes_batch_last_error(self._h).decode())
        for c, ch, m in zip(self.members, chains, samples_per_chain):
            c.chains = int(ch)
            c.ns = int(ch) * int(m)
        return emats, [x.as_dict() for x in infos], list(stat), ms.value


def footprint_bytes(n_spins, n_hidden, n_states, chains, samples_per_chain, precision=0, complex_arith=False,
                    lib=None):
    """Device bytes a context of this shape holds during SR steps (no GPU needed)."""
    lib = lib or load_library()
    out = ctypes.c_uint64()
    st = lib.nqes_footprint_bytes(int(n_spins), int(n_hidden), int(n_states), int(chains), int(samples_per_chain),
                                  int(precision), int(bool(complex_arith)), ctypes.byref(out))
    if st != OK:
        raise NqesError(st, "invalid shape")
    return out.value


class Server:
    """Serving loop: continuous batching of SR solves on one GPU (nqes_server_*)."""

    DEFAULTS = dict(h=0.595, seed=1, chains=64, samples_per_chain=100, burn_in=16, lr0=0.1, lr_decay=0.99,
                    lr_cutoff=0.01, reglam0=40.0, reglam_decay=0.9, reglam_cutoff=1.0, minres_rtol=1e-9,
                    minres_maxit=100000, tol=1e-6, max_steps=50, precision=PRECISION_FP64)

    def __init__(self, hbm_budget_bytes, max_active=64, device=0, lib=None):
        self.lib = lib or load_library()
        h_ = ctypes.c_void_p()
        st = self.lib.nqes_server_create(int(device), int(hbm_budget_bytes), int(max_active), ctypes.byref(h_))
        if st != OK:
            raise NqesError(st, self.lib.nqes_server_last_error(None).decode())
        self._h = h_
        self._keep = {}

    def submit(self, n_spins, n_hidden, n_states, J, weights=None, **kw):
        """Queues one solve; weights = (a, b, w) complex arrays or None (the reference's init). Returns its id."""
        p = dict(self.DEFAULTS)
        p.update(kw)
        Jc = np.ascontiguousarray(J, np.float64)
        r = Request()
        r.n_spins, r.n_hidden, r.n_states = int(n_spins), int(n_hidden), int(n_states)
        r.J = Jc.ctypes.data_as(_dp)
        keep = [Jc]
        if weights is not None:
            a, b, w = (np.ascontiguousarray(x, np.complex128) for x in weights)
            r.a, r.b, r.w = _cp(a), _cp(b), _cp(w)
            keep += [a, b, w]
        for k in ("h", "seed", "chains", "samples_per_chain", "burn_in", "lr0", "lr_decay", "lr_cutoff", "reglam0",
                  "reglam_decay", "reglam_cutoff", "minres_rtol", "minres_maxit", "tol", "max_steps", "precision"):
            setattr(r, k, p[k])
        rid = ctypes.c_uint64()
        st = self.lib.nqes_server_submit(self._h, ctypes.byref(r), ctypes.byref(rid))
        if st != OK:
            raise NqesError(st, self.lib.nqes_server_last_error(self._h).decode())
        return rid.value

    def poll(self, max_results=256):
        out = (Result * max_results)()
        n = ctypes.c_int()
        st = self.lib.nqes_server_poll(self._h, out, max_results, ctypes.byref(n))
        if st != OK:
            raise NqesError(st, "poll failed")
        return [out[i].as_dict() for i in range(n.value)]

    def status(self):
        q, a, d = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        b = ctypes.c_uint64()
        self.lib.nqes_server_status(self._h, ctypes.byref(q), ctypes.byref(a), ctypes.byref(d), ctypes.byref(b))
        return {"queued": q.value, "active": a.value, "done": d.value, "bytes_in_use": b.value}

    def last_error(self):
        """The last rejected submit's or failed batched step's message ('' if none)."""
        return self.lib.nqes_server_last_error(self._h).decode()

    def times(self):
        """Cumulative worker seconds by phase and the step / batch-rebuild counts."""
        v = [ctypes.c_double() for _ in range(4)]
        n = [ctypes.c_uint64() for _ in range(2)]
        self.lib.nqes_server_times(self._h, *[ctypes.byref(x) for x in v], *[ctypes.byref(x) for x in n])
        return {"admit_s": v[0].value, "rebuild_s": v[1].value, "step_s": v[2].value, "post_s": v[3].value,
                "steps": n[0].value, "rebuilds": n[1].value}

    def wait_all(self, n_expected, timeout=600.0):
        """Polls until n_expected results arrived (or timeout seconds passed)."""
        import time
        res, t0 = [], time.time()
        while len(res) < n_expected and time.time() - t0 < timeout:
            res += self.poll()
            if len(res) < n_expected:
                time.sleep(0.005)
        return res

    def close(self):
        if getattr(self, "_h", None):
            self.lib.nqes_server_destroy(self._h)
            self._h = None
