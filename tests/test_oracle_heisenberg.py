"""The oracle's Heisenberg-like local energy (its restatement of
code/rbm.cc:1091-1119, two sequential single flips per anti-aligned pair)
against the definition evaluated directly: E = Phi^-1 (H Phi) with
H = sum_{i>j} J_ij (sx_i sx_j + sy_i sy_j + delta sz_i sz_j) applied to the
amplitudes psi_kk(s) = exp(sum_i s_i a_i) prod_m cosh(b_m + sum_i s_i w_im) of
every configuration, for the hs and xxz couplings of code/rbm.cc:1064-1089."""
import numpy as np
import pytest

import helpers
from helpers import Oracle


def hs_j(n):
    """J_ij = 1 / d_ij^2, d_ij = (N / pi) sin(pi (i - j) / N), i > j."""
    J = np.zeros((n, n))
    for i in range(1, n):
        for j in range(i):
            d = np.sin(np.pi * (i - j) / n) * n / np.pi
            J[i, j] = 1.0 / (d * d)
    return J


def xxz_j(n):
    """J_ij = -1 on the bonds (i, i-1) and (N-1, 0) of the periodic chain."""
    J = np.zeros((n, n))
    for i in range(1, n):
        J[i, i - 1] = -1.0
    if n > 2:
        J[n - 1, 0] = -1.0
    return J


def sigmas(word, n):
    return np.array([-1.0 if (int(word) >> i) & 1 else 1.0 for i in range(n)])


def psi(a, b, w, s):
    """Amplitudes of every RBM kk at spins s (+-1)."""
    return np.exp(a @ s) * np.prod(np.cosh(b + np.einsum("i,kim->km", s, w)), axis=1)


def local_energy_by_definition(a, b, w, J, delta, words, n):
    K = a.shape[0]
    phi = np.array([psi(a, b, w, sigmas(words[k], n)) for k in range(K)])  # [k][kk]
    hphi = np.zeros((K, K), complex)
    for k in range(K):
        s = sigmas(words[k], n)
        for i in range(1, n):
            for j in range(i):
                if J[i, j] == 0.0:
                    continue
                hphi[k] += J[i, j] * delta * s[i] * s[j] * phi[k]
                if s[i] != s[j]:
                    sp = s.copy()
                    sp[i], sp[j] = -sp[i], -sp[j]
                    hphi[k] += 2.0 * J[i, j] * psi(a, b, w, sp)
    return np.linalg.solve(phi, hphi)


@pytest.mark.parametrize("model,N,M,K,real", [("xxz", 6, 5, 2, False), ("hs", 6, 5, 2, False), ("xxz", 5, 3, 3, True),
                                              ("hs", 7, 4, 1, True), ("hs", 66, 3, 2, False)])
def test_heisenberg_local_energy_matches_definition(model, N, M, K, real):
    J, delta = (hs_j(N), 1.0) if model == "hs" else (xxz_j(N), -1.0)
    a, b, w = helpers.random_weights(N, M, K, 0.3 if N < 20 else 0.05, 17 + N + K, real=real)
    orc = Oracle(N, M, K, J, 0.0)
    orc.set_weights(a, b, w)
    orc.set_hamiltonian(1, delta)
    rng = np.random.default_rng(N * K)
    nw = (N + 63) // 64
    for _ in range(4):
        bits = rng.integers(0, 2, size=(K, N))
        full = [sum(int(bits[k, i]) << i for i in range(N)) for k in range(K)]
        words = np.array([[(full[k] >> (64 * t)) & ((1 << 64) - 1) for t in range(nw)] for k in range(K)],
                         dtype=np.uint64)
        E, _ = orc.local(words)
        ref = local_energy_by_definition(a, b, w, J, delta, full, N)
        assert np.max(np.abs(E - ref)) / np.max(np.abs(ref)) < 1e-11
