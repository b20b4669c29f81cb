"""The oracle's SR step (its restatement of code/rbm.cc:574-719) against the
formulas evaluated directly from its per-sample local energies E_s and
log-derivatives O_s (which tests/test_oracle.py pins to their definitions):
  e_mat = <E>;  o = <O>;  skk = reglam (<|O|^2> - |o|^2);
  f = <tr(E) conj(O)> - <tr E> conj(o)                      (code/rbm.cc:640-650)
  (S v)_l = <conj(O_l) (O . v)> + skk_l v_l - (o . v) conj(o_l)  (code/rbm.cc:660-683)
and the update w -= lr x with x the MINRES-QLP solution of S x = f, checked by
its residual against the dense S (code/rbm.cc:699-717)."""
import numpy as np
import pytest

import helpers
from helpers import Oracle, synthetic_j


def p_layout(a, b, w):
    """Weights in the log-derivative layout [k][a_i | b_j | w_{i*M+j}]."""
    K = a.shape[0]
    return np.concatenate([np.concatenate([a[k].ravel(), b[k].ravel(), w[k].ravel()]) for k in range(K)])


@pytest.mark.parametrize("N,M,K,real", [(4, 8, 2, False), (5, 6, 3, True), (6, 4, 1, False)])
def test_sr_step_matches_formulas(N, M, K, real):
    orc = Oracle(N, M, K, synthetic_j(N), 0.7)
    w0 = helpers.random_weights(N, M, K, 0.1, 13 + N, real=real)
    orc.set_weights(*w0)
    C, m, burn, lr, reglam = 6, 12, 4, 0.1, 3.0
    emat, info = orc.sr_step(77 + N, C, m, burn, lr, reglam, 1e-12, 5000)
    ns = C * m
    spins, eloc, E = orc.samples(ns)
    O = np.array([orc.sample_deriv(s) for s in range(ns)])
    assert np.allclose(eloc, np.trace(E, axis1=1, axis2=2), rtol=1e-13, atol=1e-13)
    assert np.max(np.abs(emat - E.mean(axis=0))) <= 1e-12 * np.max(np.abs(emat))
    o = O.mean(axis=0)
    skk = reglam * ((np.abs(O) ** 2).mean(axis=0) - np.abs(o) ** 2)
    el = eloc.mean()
    f = (eloc[:, None] * np.conj(O)).mean(axis=0) - el * np.conj(o)
    go, gs, gf = orc.moments()
    assert np.max(np.abs(go - o)) <= 1e-12 * np.max(np.abs(o))
    assert np.max(np.abs(gs - skk)) <= 1e-11 * np.max(np.abs(skk))
    assert np.max(np.abs(gf - f)) <= 1e-11 * np.max(np.abs(f))
    S = (np.conj(O).T @ O) / ns + np.diag(skk) - np.outer(np.conj(o), o)
    rng = np.random.default_rng(N)
    v = rng.normal(size=orc.P) + 1j * rng.normal(size=orc.P)
    assert np.max(np.abs(orc.apply_S(v) - S @ v)) <= 1e-11 * np.max(np.abs(S @ v))
    x = (p_layout(*w0) - p_layout(*orc.get_weights())) / lr
    assert np.linalg.norm(S @ x - f) <= 1e-8 * (np.linalg.norm(S, 2) * np.linalg.norm(x) + np.linalg.norm(f))
