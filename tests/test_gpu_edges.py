"""Edge cases of the SR step against the oracle: the largest shape the library
accepts (N = 128 spins, M = 512 hidden units, K = 4 states), one chain with one
sample and no burn-in, the smallest networks (N = 1, 2; M = 1), an iteration
cap that stops MINRES-QLP after one step, and invalid step arguments.

Tolerances are those of the FP64 parity tests: configurations and accept
counts bit-exact, amplitudes, energies, moments and S·v within 1e-11
relative; weight updates within 1e-6 (1e-9 after a single MINRES-QLP
iteration). The 20-iteration capped solve at the largest shape is checked by
its residual instead: there the iterate itself depends on rounding."""
import numpy as np
import pytest

import __graft_entry__ as ge
import helpers
from helpers import Oracle, synthetic_j

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def flat(ws):
    return np.concatenate([x.ravel() for x in ws])


def step_both(pkg, N, M, K, real, scale, wseed, args):
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, scale, wseed, real=real)
    ctx = pkg.Context(N, M, K, J, 0.595)
    ctx.set_weights(*w)
    orc = Oracle(N, M, K, J, 0.595)
    orc.set_weights(*w)
    e_g, info = ctx.sr_step(*args)
    e_o, oinfo = orc.sr_step(*args)
    return ctx, orc, w, (e_g, info), (e_o, oinfo)


def check_step(ctx, orc, w, g, o, ns, dw_tol):
    (e_g, info), (e_o, oinfo) = g, o
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
    if int(oinfo["flag"]) == 8:  # stopped by the iteration cap
        assert it_g == it_o
    else:  # a stopping test near its threshold may go either way by an iteration
        assert abs(it_g - it_o) <= 1, (it_g, it_o)
    w0 = flat(w)
    dg, do = flat(ctx.get_weights()) - w0, flat(orc.get_weights()) - w0
    if np.max(np.abs(do)) == 0.0:
        assert np.max(np.abs(dg)) == 0.0
    elif dw_tol is not None:
        assert rel_err(dg, do) < dw_tol
    else:
        # Iterates of a capped solve of an ill-conditioned system depend on
        # rounding (the oracle's own iterate changes with its thread count);
        # what both solvers guarantee is the residual they report.
        x = ctx.get_solution()
        f = orc.moments()[2]
        r = np.linalg.norm(orc.apply_S(x) - f) / (info["anorm"] * np.linalg.norm(x) + np.linalg.norm(f))
        assert r <= 2.0 * max(info["relres"], oinfo["relres"]), (r, info["relres"], oinfo["relres"])
        assert 0.5 < info["relres"] / oinfo["relres"] < 2.0, (info["relres"], oinfo["relres"])


@pytest.mark.parametrize("real", [True, False])
def test_largest_shape(pkg, real):
    """N = 128 (two full configuration words), M = 512, K = 4: the shared-memory
    layout of the complex sampler is within 48 bytes of the 227 KB limit. The
    solve is capped at 20 iterations (flag 8) to keep the oracle's dense
    P = 264,704 passes short."""
    N, M, K = 128, 512, 4
    chains, m, burn = (2, 3, 1) if real else (1, 2, 1)
    ctx, orc, w, g, o = step_both(pkg, N, M, K, real, 0.02, 5, (77, chains, m, burn, 0.1, 2.0, 1e-9, 20))
    assert int(g[1]["minres_flag"]) == 8
    check_step(ctx, orc, w, g, o, chains * m, None)
    v = np.random.default_rng(2).normal(size=ctx.P) + (0 if real else 1j) * np.random.default_rng(3).normal(size=ctx.P)
    assert rel_err(ctx.apply_S(v), orc.apply_S(v)) < 1e-11
    for s in (0, chains * m - 1):
        assert rel_err(ctx.get_O(s, 1)[0], orc.sample_deriv(s)) < 1e-11
    ctx.close()


def test_largest_shape_mixed_and_certified(pkg):
    """At N = 128, M = 512, K = 4 the mixed form (block sampler, factored S·v)
    and the certified form keep the FP64 chains bit for bit."""
    N, M, K, chains, m = 128, 512, 4, 4, 4
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.02, 9, real=True)
    out = {}
    for prec in (pkg.PRECISION_FP64, pkg.PRECISION_MIXED, pkg.PRECISION_CERTIFIED):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_PRECISION, prec)
        e, info = ctx.sr_step(31, chains, m, 2, 0.1, 5.0, 1e-9, 30)
        spins, _, E = ctx.get_samples()
        out[prec] = dict(e=e, spins=spins, E=E, acc=ctx.get_accepts())
        ctx.close()
    f = out[pkg.PRECISION_FP64]
    for prec, tol in ((pkg.PRECISION_MIXED, 1e-5), (pkg.PRECISION_CERTIFIED, 1e-11)):
        x = out[prec]
        assert np.array_equal(f["spins"], x["spins"]), prec
        assert np.array_equal(f["acc"], x["acc"]), prec
        assert rel_err(x["E"], f["E"]) < tol
        assert rel_err(x["e"], f["e"]) < tol


@pytest.mark.parametrize("real", [True, False])
def test_one_chain_one_sample(pkg, real):
    """One chain, one sample, no burn-in: the centred moments vanish, so both
    S (its regularised diagonal included) and the force are zero up to
    rounding. The oracle's force is exactly zero and it stops at iteration 0;
    in complex arithmetic the GPU's E O* - E O* can leave 1e-16 of E |O|, and
    a solve of rounding noise against rounding noise is noise in any
    implementation, so the update is compared only where the force is zero."""
    N, M, K = 8, 16, 2
    ctx, orc, w, (e_g, info), (e_o, oinfo) = step_both(pkg, N, M, K, real, 0.1, 21,
                                                       (5, 1, 1, 0, 0.1, 2.0, 1e-9, 1000))
    assert int(oinfo["iters"]) == 0
    sg, _, Eg = ctx.get_samples()
    so, _, Eo = orc.samples(1)
    assert np.array_equal(sg, so) and info["accepted"] == oinfo["accepted"]
    assert rel_err(Eg, Eo) < 1e-11 and rel_err(e_g, e_o) < 1e-11
    (og, sg_, fg), (oo, so_, fo) = ctx.get_moments(), orc.moments()
    assert rel_err(og, oo) < 1e-11 and rel_err(sg_, so_) < 1e-10
    assert np.max(np.abs(fo)) == 0.0
    assert np.max(np.abs(fg)) <= 1e-14 * np.max(np.abs(Eo)) * np.max(np.abs(oo))
    w0 = flat(w)
    assert np.array_equal(flat(orc.get_weights()), w0)
    if np.max(np.abs(fg)) == 0.0:
        assert int(info["minres_iters"]) == 0 and np.array_equal(flat(ctx.get_weights()), w0)
    ctx.close()


def test_one_chain_one_sample_mixed(pkg):
    """The mixed and certified forms at one chain and one sample keep the FP64
    chain and energies."""
    N, M, K = 8, 16, 2
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.1, 21, real=True)
    res = []
    for prec in (pkg.PRECISION_FP64, pkg.PRECISION_MIXED, pkg.PRECISION_CERTIFIED):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_PRECISION, prec)
        e, info = ctx.sr_step(5, 1, 1, 0, 0.1, 2.0, 1e-9, 1000)
        res.append((ctx.get_samples()[0], e))
        ctx.close()
    for s, e in res:
        assert np.array_equal(s, res[0][0])
        assert rel_err(e, res[0][1]) < 1e-6


@pytest.mark.parametrize("N,M,K,real", [(1, 1, 1, True), (2, 1, 1, False), (3, 2, 1, True)])
def test_smallest_networks(pkg, N, M, K, real):
    """One or two spins and one hidden unit: a single configuration word with
    31 idle lanes, and for N = 1 no Ising term at all."""
    ctx, orc, w, g, o = step_both(pkg, N, M, K, real, 0.3, 13 + N, (40 + N, 3, 5, 2, 0.1, 2.0, 1e-9, 100))
    check_step(ctx, orc, w, g, o, 15, 1e-6)
    ctx.close()


def test_iteration_cap_of_one(pkg):
    """maxit = 1: both solvers stop after one iteration with flag 8 and take
    the same step."""
    ctx, orc, w, g, o = step_both(pkg, 8, 16, 2, True, 0.1, 4, (61, 4, 6, 2, 0.1, 2.0, 1e-9, 1))
    assert int(o[1]["flag"]) == 8 and int(o[1]["iters"]) == 1
    check_step(ctx, orc, w, g, o, 24, 1e-9)
    ctx.close()


def test_invalid_step_arguments_leave_the_context_usable(pkg):
    """Invalid counts, burn-in, tolerance or non-finite schedule values are
    rejected before any launch; the next valid step gives the results of a
    fresh context."""
    N, M, K = 8, 16, 2
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.1, 8, real=True)
    ctx = pkg.Context(N, M, K, J, 0.595)
    ctx.set_weights(*w)
    good = (12, 4, 5, 2, 0.1, 2.0, 1e-9, 100)
    for bad in [(12, 0, 5, 2, 0.1, 2.0, 1e-9, 100), (12, 4, 0, 2, 0.1, 2.0, 1e-9, 100),
                (12, 4, 5, -1, 0.1, 2.0, 1e-9, 100), (12, 4, 5, 2, float("nan"), 2.0, 1e-9, 100),
                (12, 4, 5, 2, 0.1, float("inf"), 1e-9, 100), (12, 4, 5, 2, 0.1, 2.0, -1.0, 100)]:
        with pytest.raises(pkg.NqesError) as err:
            ctx.sr_step(*bad)
        assert err.value.status == pkg.ERR_INVALID
    e1, _ = ctx.sr_step(*good)
    s1 = ctx.get_samples()[0]
    ctx.close()
    ref = pkg.Context(N, M, K, J, 0.595)
    ref.set_weights(*w)
    e2, _ = ref.sr_step(*good)
    assert np.array_equal(e1, e2) and np.array_equal(s1, ref.get_samples()[0])
    ref.close()


def psi_all(a, b, w, s):
    return np.exp(a @ s) * np.prod(np.cosh(b + np.einsum("i,kim->km", s, w)), axis=1)


def sig(v, n):
    return np.array([-1.0 if (v >> i) & 1 else 1.0 for i in range(n)])


@pytest.mark.parametrize("N,M,K,rows", [(6, 8, 2, (5, 5)), (5, 6, 3, (9, 3, 9)), (7, 5, 4, (1, 1, 1, 1))])
def test_evaluate_singular_phi_uses_the_pseudo_inverse(pkg, N, M, K, rows):
    """Evaluation at configurations with equal rows (Phi singular), as the
    reference's --dump-ham enumerates them: E = Phi^+ (H Phi) with the
    Moore-Penrose pseudo-inverse (code/rbm.cc:1159-1164), here against numpy's
    pinv of the brute-force H Phi; O is zero (det(Phi^+ Phi~) of a
    rank-deficient product)."""
    J = synthetic_j(N)
    h = 0.7
    a, b, w = helpers.random_weights(N, M, K, 0.3, 3 + N, real=False)
    ctx = pkg.Context(N, M, K, J, h)
    ctx.set_weights(a, b, w)
    cfg = np.array([[[r] for r in rows]], dtype=np.uint64)
    phi, _, E, O = ctx.evaluate(cfg)
    ctx.close()
    S = [sig(r, N) for r in rows]
    Phi = np.array([psi_all(a, b, w, S[k]) for k in range(K)])
    assert rel_err(phi[0], Phi) < 1e-12
    HPhi = np.zeros((K, K), complex)
    for k in range(K):
        s = S[k]
        jt = sum(J[i, j] * s[i] * s[j] for i in range(N) for j in range(i))
        HPhi[k] = 2.0 * jt * Phi[k]
        for i in range(N):
            sp = s.copy()
            sp[i] = -sp[i]
            HPhi[k] -= h * psi_all(a, b, w, sp)
    Eref = np.linalg.pinv(Phi) @ HPhi
    assert rel_err(E[0], Eref) < 1e-10
    assert np.max(np.abs(O)) <= 1e-12 * max(1.0, np.max(np.abs(Phi)))


def test_staging_wait_runs_out_and_reports_timeout(pkg):
    """A bounded device-side wait that runs out is reported, not hung: with the
    test hook, the sampler's table staging waits for bytes that no copy
    delivers (nothing is in flight), gives up after its poll limit, and the
    step returns NQES_ERR_TIMEOUT. The context stays usable: with the hook off
    its next step equals a fresh context's."""
    N, M, K = 32, 64, 2
    w = pkg.synthetic_weights(N, M, K, 0.01, 5)

    def make():
        c = pkg.Context(N, M, K, synthetic_j(N), 0.595)
        c.set_weights(*w)
        c.set_option(pkg.OPT_PRECISION, pkg.PRECISION_MIXED)
        c.set_option(pkg.OPT_MINRES_CAP, 5)
        return c

    ctx = make()
    ctx.set_option(pkg.OPT_TEST_STAGE_WAIT, 1)
    with pytest.raises(pkg.NqesError) as e:
        ctx.sr_step(7, 16, 4, 2, 0.0, 5.0, 1e-9, 100)
    assert e.value.status == pkg.ERR_TIMEOUT
    assert "wait ran out" in str(e.value)
    ctx.set_option(pkg.OPT_TEST_STAGE_WAIT, 0)
    ctx.set_weights(*w)
    got, _ = ctx.sr_step(9, 16, 4, 2, 0.1, 5.0, 1e-9, 100)
    ref = make()
    want, _ = ref.sr_step(9, 16, 4, 2, 0.1, 5.0, 1e-9, 100)
    assert np.array_equal(got, want)
    assert np.array_equal(ctx.get_samples()[0], ref.get_samples()[0])
    ctx.close()
    ref.close()
