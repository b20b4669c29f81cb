"""The oracle's correlation stage (its restatement of code/rbm.cc:728-826)
against the definitions evaluated directly on the same Markov chains: for every
sample s of chain c (pcg64(seed + c), burn-in then one sample per sweep) the
K×K matrices Phi(s)^-1 F_i(s) with
  x_i:   F = Phi(s with spin i flipped in every row)        (corrfcn_x)
  z_i:   F = Phi(s) with row k negated where spin i is down (corrfcn_z)
  xx_ij: F = Phi(s with spins i and j flipped in every row) (corrfcn_xx)
  zz_ij: F = Phi(s) with row k negated where s_i != s_j     (corrfcn_zz)
averaged over all samples, then diag(V^-1 mean V).real. Amplitudes
psi_kk(s) = exp(sum_i s_i a_i) prod_m cosh(b_m + sum_i s_i w_im) come from
numpy here, independently of the oracle's incremental updates."""
import numpy as np
import pytest

import helpers
from helpers import Oracle, synthetic_j


def sigmas(word, n):
    return np.array([-1.0 if (int(word) >> i) & 1 else 1.0 for i in range(n)])


def phi_of(a, b, w, S):
    """Phi[k][kk] = psi_kk(S[k])."""
    return np.array([np.exp(a @ s) * np.prod(np.cosh(b + np.einsum("i,kim->km", s, w)), axis=1) for s in S])


@pytest.mark.parametrize("N,M,K,real", [(6, 5, 2, False), (5, 4, 3, True), (7, 3, 1, False)])
def test_correlations_match_definitions(N, M, K, real):
    a, b, w = helpers.random_weights(N, M, K, 0.3, 41 + N, real=real)
    J = synthetic_j(N)
    orc = Oracle(N, M, K, J, 0.8)
    orc.set_weights(a, b, w)
    rng = np.random.default_rng(K)
    V = rng.normal(size=(K, K)) + 1j * rng.normal(size=(K, K)) + 2.0 * np.eye(K)
    seed, C, m, burn = 900 + N, 3, 4, 2
    x, z, xx, zz = orc.correlations(seed, C, m, burn, V, threads=1)

    acc = {"x": np.zeros((N, K, K), complex), "z": np.zeros((N, K, K), complex),
           "xx": np.zeros((N * N, K, K), complex), "zz": np.zeros((N * N, K, K), complex)}
    for c in range(C):
        spins = orc.chain(seed + c, burn + m)[0]
        for t in range(burn, burn + m):
            S = [sigmas(spins[t, k, 0], N) for k in range(K)]
            Phi = phi_of(a, b, w, S)
            Pinv = np.linalg.inv(Phi)
            for i in range(N):
                Sx = [s.copy() for s in S]
                for s in Sx:
                    s[i] = -s[i]
                acc["x"][i] += Pinv @ phi_of(a, b, w, Sx)
                Fz = Phi * np.array([[-1.0 if S[k][i] < 0 else 1.0] for k in range(K)])
                acc["z"][i] += Pinv @ Fz
                for j in range(N):
                    Sxx = [s.copy() for s in S]
                    for s in Sxx:
                        s[i] = -s[i]
                        s[j] = -s[j]
                    acc["xx"][i * N + j] += Pinv @ phi_of(a, b, w, Sxx)
                    Fzz = Phi * np.array([[-1.0 if S[k][i] != S[k][j] else 1.0] for k in range(K)])
                    acc["zz"][i * N + j] += Pinv @ Fzz
    Vinv = np.linalg.inv(V)
    for name, got in (("x", x), ("z", z), ("xx", xx), ("zz", zz)):
        mats = acc[name] / (C * m)
        want = np.array([np.diag(Vinv @ mt @ V).real for mt in mats])
        assert np.max(np.abs(got - want)) <= 1e-10 * max(1.0, np.max(np.abs(want))), name
