"""Shared test helpers: the CPU oracle's ctypes binding, configuration packing,
and the seeded synthetic inputs the tests and the bench use."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")

_u64p = ctypes.POINTER(ctypes.c_uint64)
_dp = ctypes.POINTER(ctypes.c_double)


def dptr(a):
    return None if a is None else a.ctypes.data_as(_dp)


def uptr(a):
    return None if a is None else a.ctypes.data_as(_u64p)


def build_oracle():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)
    return os.path.join(ORACLE_DIR, "liboracle.so")


_ORACLE = None


def oracle_lib():
    global _ORACLE
    if _ORACLE is None:
        lib = ctypes.CDLL(build_oracle())
        vp, i, d, u64 = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_uint64
        sig = {
            "orc_create": (vp, [i, i, i, _dp, d]),
            "orc_set_hamiltonian": (None, [vp, i, d]),
            "orc_destroy": (None, [vp]),
            "orc_set_weights": (None, [vp, _dp, _dp, _dp]),
            "orc_get_weights": (None, [vp, _dp, _dp, _dp]),
            "orc_init_weights": (None, [vp, u64]),
            "orc_state": (None, [vp, _u64p, _dp, _dp]),
            "orc_local": (i, [vp, _u64p, _dp, _dp]),
            "orc_sr_step": (i, [vp, u64, i, i, i, d, d, d, u64, i, _dp, _dp, i]),
            "orc_samples": (None, [vp, _u64p, _dp, _dp]),
            "orc_moments": (None, [vp, _dp, _dp, _dp]),
            "orc_sample_deriv": (None, [vp, i, _dp]),
            "orc_apply_S": (None, [vp, _dp, _dp, i]),
            "orc_correlations": (None, [vp, u64, i, i, i, _dp, _dp, _dp, _dp, _dp, i]),
            "orc_chain": (None, [vp, u64, i, _u64p, _u64p]),
            "orc_pcg64": (None, [u64, i, _u64p]),
            "orc_uniform": (None, [u64, i, _dp]),
            "orc_bernoulli": (None, [u64, i, ctypes.POINTER(ctypes.c_uint8)]),
            "orc_minresqlp_dense": (i, [i, _dp, _dp, d, u64, _dp, _dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _ORACLE = lib
    return _ORACLE


def cplx_arr(flat):
    a = np.asarray(flat, dtype=np.float64)
    return a.view(np.complex128)


def cfg_words(cfgs, n):
    """Python ints (bit i = spin i down) -> K x ceil(n/64) uint64 words."""
    nw = (n + 63) // 64
    out = np.zeros((len(cfgs), nw), dtype=np.uint64)
    for k, c in enumerate(cfgs):
        c = int(c)
        for t in range(nw):
            out[k, t] = (c >> (64 * t)) & 0xFFFFFFFFFFFFFFFF
    return out


class Oracle:
    """Thin wrapper over the oracle's extern "C" functions."""

    def __init__(self, N, M, K, J, h):
        self.lib = oracle_lib()
        self.N, self.M, self.K = N, M, K
        self.L = N + M + N * M
        self.P = K * self.L
        self.NW = (N + 63) // 64
        self._J = np.ascontiguousarray(J, dtype=np.float64)
        self.h = ctypes.c_void_p(self.lib.orc_create(N, M, K, dptr(self._J), float(h)))

    def __del__(self):
        try:
            self.lib.orc_destroy(self.h)
        except Exception:
            pass

    def set_hamiltonian(self, form, delta=0.0):
        self.lib.orc_set_hamiltonian(self.h, int(form), float(delta))

    def set_weights(self, a, b, w):
        a = np.ascontiguousarray(a, np.complex128)
        b = np.ascontiguousarray(b, np.complex128)
        w = np.ascontiguousarray(w, np.complex128)
        self.lib.orc_set_weights(self.h, dptr(a.view(np.float64)), dptr(b.view(np.float64)),
                                 dptr(w.view(np.float64)))

    def get_weights(self):
        a = np.zeros((self.K, self.N), np.complex128)
        b = np.zeros((self.K, self.M), np.complex128)
        w = np.zeros((self.K, self.N, self.M), np.complex128)
        self.lib.orc_get_weights(self.h, dptr(a.view(np.float64)), dptr(b.view(np.float64)),
                                 dptr(w.view(np.float64)))
        return a, b, w

    def init_weights(self, seed):
        self.lib.orc_init_weights(self.h, seed)

    def state(self, words):
        K, M = self.K, self.M
        phi = np.zeros(K * K, np.complex128)
        th = np.zeros(M * K * K, np.complex128)
        w = np.ascontiguousarray(words, np.uint64)
        self.lib.orc_state(self.h, uptr(w), dptr(phi.view(np.float64)), dptr(th.view(np.float64)))
        return phi.reshape(K, K), th.reshape(M, K * K)

    def local(self, words):
        E = np.zeros(self.K * self.K, np.complex128)
        O = np.zeros(self.P, np.complex128)
        w = np.ascontiguousarray(words, np.uint64)
        rc = self.lib.orc_local(self.h, uptr(w), dptr(E.view(np.float64)), dptr(O.view(np.float64)))
        assert rc == 0
        return E.reshape(self.K, self.K), O

    def sr_step(self, seed, chains, m, burn, lr, reglam, rtol, maxit, store_o=False, threads=0):
        emat = np.zeros(self.K * self.K, np.complex128)
        info = np.zeros(9)
        threads = threads or os.cpu_count()
        self.lib.orc_sr_step(self.h, seed, chains, m, burn, lr, reglam, rtol, maxit, int(store_o),
                             dptr(emat.view(np.float64)), dptr(info), threads)
        keys = ["flag", "iters", "qlp_iters", "relres", "anorm", "acond", "xnorm", "accepted", "singular"]
        return emat.reshape(self.K, self.K), dict(zip(keys, info.tolist()))

    def samples(self, ns):
        spins = np.zeros((ns, self.K, self.NW), np.uint64)
        eloc = np.zeros(ns, np.complex128)
        emat = np.zeros((ns, self.K, self.K), np.complex128)
        self.lib.orc_samples(self.h, uptr(spins), dptr(eloc.view(np.float64)), dptr(emat.view(np.float64)))
        return spins, eloc, emat

    def moments(self):
        o = np.zeros(self.P, np.complex128)
        s = np.zeros(self.P, np.complex128)
        f = np.zeros(self.P, np.complex128)
        self.lib.orc_moments(self.h, dptr(o.view(np.float64)), dptr(s.view(np.float64)), dptr(f.view(np.float64)))
        return o, s, f

    def sample_deriv(self, s):
        out = np.zeros(self.P, np.complex128)
        self.lib.orc_sample_deriv(self.h, s, dptr(out.view(np.float64)))
        return out

    def apply_S(self, v, threads=0):
        v = np.ascontiguousarray(v, np.complex128)
        out = np.zeros(self.P, np.complex128)
        self.lib.orc_apply_S(self.h, dptr(v.view(np.float64)), dptr(out.view(np.float64)),
                             threads or os.cpu_count())
        return out

    def correlations(self, seed, chains, m, burn, evecs, threads=0):
        N, K = self.N, self.K
        ev = np.ascontiguousarray(evecs, np.complex128)
        x = np.zeros((N, K))
        z = np.zeros((N, K))
        xx = np.zeros((N * N, K))
        zz = np.zeros((N * N, K))
        self.lib.orc_correlations(self.h, seed, chains, m, burn, dptr(ev.view(np.float64)), dptr(x), dptr(z),
                                  dptr(xx), dptr(zz), threads or os.cpu_count())
        return x, z, xx, zz

    def chain(self, seed, sweeps):
        spins = np.zeros((sweeps, self.K, self.NW), np.uint64)
        acc = np.zeros((sweeps, self.K * self.N), np.uint64)
        self.lib.orc_chain(self.h, seed, sweeps, uptr(spins), uptr(acc))
        return spins, acc


def synthetic_j(n, alpha=1.2):
    """J_ij = |i-j|^-alpha for i != j, zero diagonal, max |J| = 1."""
    i = np.arange(n)
    d = np.abs(i[:, None] - i[None, :]).astype(float)
    with np.errstate(divide="ignore"):
        J = np.where(d > 0, d ** (-alpha), 0.0)
    return J / np.max(np.abs(J)) if n > 1 else J


def random_weights(N, M, K, scale, seed, real=False):
    rng = np.random.default_rng(seed)
    def draw(shape):
        z = rng.normal(size=shape) * scale
        if not real:
            z = z + 1j * rng.normal(size=shape) * scale
        return z.astype(np.complex128)
    return draw((K, N)), draw((K, M)), draw((K, N, M))
