"""The oracle's Markov chain (its restatement of code/rbm.cc:98-119, 530-552)
replayed from the definitions: the start configuration from K·N Bernoulli(1/2)
draws (k-major, bit set = spin down), then per sweep the proposals k outer,
i inner, each taking the next uniform u of the same pcg64 stream (every draw of
either distribution consumes one 64-bit output; the streams are pinned to the
reference's pcg_random.h and libstdc++ in test_oracle.py) and accepted iff
u <= min(1, |det Phi'|^2 / |det Phi|^2), with Phi from numpy amplitudes
psi_kk(s) = exp(sum_i s_i a_i) prod_m cosh(b_m + sum_i s_i w_im)."""
import ctypes

import numpy as np
import pytest

import helpers
from helpers import Oracle, dptr, oracle_lib, synthetic_j


def phi_of(a, b, w, words, n):
    S = [np.array([-1.0 if (int(v) >> i) & 1 else 1.0 for i in range(n)]) for v in words]
    return np.array([np.exp(a @ s) * np.prod(np.cosh(b + np.einsum("i,kim->km", s, w)), axis=1) for s in S])


@pytest.mark.parametrize("N,M,K,real", [(6, 5, 2, False), (5, 4, 3, True), (7, 6, 1, False), (4, 3, 4, False)])
def test_chain_matches_definition(N, M, K, real):
    a, b, w = helpers.random_weights(N, M, K, 0.3, 61 + N + K, real=real)
    orc = Oracle(N, M, K, synthetic_j(N), 0.5)
    orc.set_weights(a, b, w)
    seed, sweeps = 4242 + N, 8
    spins, acc = orc.chain(seed, sweeps)
    lib = oracle_lib()
    KN = K * N
    bern = np.zeros(KN, np.uint8)
    lib.orc_bernoulli(seed, KN, bern.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    u = np.zeros(KN + sweeps * KN)
    lib.orc_uniform(seed, len(u), dptr(u))
    cfg = [sum(int(bern[k * N + i]) << i for i in range(N)) for k in range(K)]
    t = KN
    checked = 0
    for sw in range(sweeps):
        for k in range(K):
            for i in range(N):
                d0 = np.linalg.det(phi_of(a, b, w, cfg, N))
                prop = list(cfg)
                prop[k] ^= 1 << i
                d1 = np.linalg.det(phi_of(a, b, w, prop, N))
                prob = 1.0 if d0 == 0 else abs(d1) ** 2 / abs(d0) ** 2
                want = u[t] <= min(1.0, prob)
                got = bool(acc[sw, k * N + i])
                if abs(u[t] - prob) > 1e-9 * max(prob, 1e-300):  # away from a tie the decision is defined
                    assert got == want, (sw, k, i, u[t], prob)
                    checked += 1
                if got:
                    cfg = prop
                t += 1
        assert [int(spins[sw, k, 0]) for k in range(K)] == cfg
    assert checked >= sweeps * KN - 2
