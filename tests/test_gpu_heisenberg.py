"""GPU parity of the Heisenberg-like local energy (hs and xxz,
code/rbm.cc:1064-1119) against the oracle: the GPU forms each anti-aligned
pair's two-flip ratio in one product (cosh(d_i + d_j) - tanh sinh(d_i + d_j)
per hidden unit, from the cosh/sinh tables), the oracle takes the reference's
two sequential single flips; both FP64, so E agrees to 1e-11 relative. The
sampler does not depend on the Hamiltonian: configurations and accept counts
stay bit-exact."""
import numpy as np
import pytest

import __graft_entry__ as ge
import helpers
from helpers import Oracle
from test_oracle_heisenberg import hs_j, xxz_j

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def model_j(model, n):
    return (hs_j(n), 1.0) if model == "hs" else (xxz_j(n), -1.0)


def make_pair(pkg, model, N, M, K, scale, seed, real):
    J, delta = model_j(model, N)
    a, b, w = helpers.random_weights(N, M, K, scale, seed, real=real)
    ctx = pkg.Context(N, M, K, J, 0.0)
    ctx.set_weights(a, b, w)
    ctx.set_hamiltonian(pkg.HAM_HEISENBERG_LIKE, delta)
    orc = Oracle(N, M, K, J, 0.0)
    orc.set_weights(a, b, w)
    orc.set_hamiltonian(1, delta)
    return ctx, orc


@pytest.mark.parametrize("model,N,M,K,real", [("xxz", 10, 8, 2, False), ("hs", 10, 8, 2, True),
                                              ("hs", 70, 12, 3, False)])
def test_evaluate_matches_oracle(pkg, model, N, M, K, real):
    ctx, orc = make_pair(pkg, model, N, M, K, 0.2 if N < 20 else 0.03, 5 + N, real)
    rng = np.random.default_rng(N + K)
    nw = (N + 63) // 64
    bits = rng.integers(0, 2, size=(6, K, N))
    cfgs = np.zeros((6, K, nw), np.uint64)
    for c in range(6):
        for k in range(K):
            v = sum(int(bits[c, k, i]) << i for i in range(N))
            for t in range(nw):
                cfgs[c, k, t] = np.uint64((v >> (64 * t)) & ((1 << 64) - 1))
    _, _, E, O = ctx.evaluate(cfgs)
    for c in range(6):
        oE, oO = orc.local(cfgs[c])
        assert rel_err(E[c], oE) < 1e-11
        assert rel_err(O[c], oO) < 1e-11
    ctx.close()


@pytest.mark.parametrize("model,N,M,K,real", [("xxz", 8, 16, 2, True), ("hs", 8, 16, 2, False),
                                              ("xxz", 12, 6, 3, False), ("hs", 33, 20, 2, True)])
def test_sr_step_parity(pkg, model, N, M, K, real):
    ctx, orc = make_pair(pkg, model, N, M, K, 0.1 if N < 20 else 0.03, 11 + N + K, real)
    chains, m, burn = (6, 12, 5) if N < 20 else (3, 6, 2)
    args = (7000 + N, chains, m, burn, 0.1, 2.0, 1e-9, 1000)
    e_g, info = ctx.sr_step(*args)
    e_o, oinfo = orc.sr_step(*args)
    ns = chains * m
    sg, _, Eg = ctx.get_samples()
    so, _, Eo = orc.samples(ns)
    assert np.array_equal(sg, so), "sampled configurations differ"
    assert info["accepted"] == oinfo["accepted"]
    assert rel_err(Eg, Eo) < 1e-11
    assert rel_err(e_g, e_o) < 1e-11
    for a, b in zip(ctx.get_moments(), orc.moments()):
        assert rel_err(a, b) < 1e-10
    assert info["minres_flag"] == int(oinfo["flag"])
    it_g, it_o = int(info["minres_iters"]), int(oinfo["iters"])
    assert abs(it_g - it_o) <= max(2, it_o // 10), (it_g, it_o)
    x = ctx.get_solution()
    fo = orc.moments()[2]
    r = np.linalg.norm(orc.apply_S(x) - fo)
    assert r <= 10 * 1e-9 * (info["anorm"] * np.linalg.norm(x) + np.linalg.norm(fo)), r
    ctx.close()


def test_heisenberg_runs_in_the_fp64_form_only(pkg):
    ctx, _ = make_pair(pkg, "xxz", 8, 16, 2, 0.1, 3, True)
    ctx.set_option(pkg.OPT_PRECISION, pkg.PRECISION_MIXED)
    with pytest.raises(pkg.NqesError) as err:
        ctx.sr_step(1, 4, 4, 2, 0.1, 2.0, 1e-9, 100)
    assert err.value.status == pkg.ERR_INVALID
    ctx.set_option(pkg.OPT_PRECISION, pkg.PRECISION_FP64)
    ctx.sr_step(1, 4, 4, 2, 0.1, 2.0, 1e-9, 100)
    ctx.set_hamiltonian(pkg.HAM_ISING_LIKE)  # and back: the ising-like form with the same context
    ctx.sr_step(2, 4, 4, 2, 0.1, 2.0, 1e-9, 100)
    ctx.close()
