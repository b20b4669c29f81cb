"""GPU parity of libnqes against the CPU oracle (restatement of code/rbm.cc).

Tolerances (FP64): amplitudes, tanh(theta), local energies, log-derivatives,
moments and S·v agree to 1e-11 relative (the oracle multiplies factors in the
reference's sequential order, the GPU in a tree; both are FP64). Random
draws, start configurations and every sampled spin configuration are
bit-exact, and so are per-chain accept counts. MINRES-QLP solutions agree to
the solver tolerance scale (1e-7 relative at rtol 1e-9)."""
import json
import os

import numpy as np
import pytest

import __graft_entry__ as ge
import helpers
from helpers import GOLDEN, Oracle, cfg_words, cplx_arr, synthetic_j

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def make_pair(pkg, N, M, K, h, scale, seed, real):
    J = synthetic_j(N)
    a, b, w = helpers.random_weights(N, M, K, scale, seed, real=real)
    ctx = pkg.Context(N, M, K, J, h)
    ctx.set_weights(a, b, w)
    orc = Oracle(N, M, K, J, h)
    orc.set_weights(a, b, w)
    return ctx, orc


def test_evaluate_matches_definitions_and_oracle(pkg):
    with open(os.path.join(GOLDEN, "physics_golden.json")) as f:
        phys = json.load(f)
    for case in phys["cases"]:
        N, M, K = case["N"], case["M"], case["K"]
        J = np.array(case["J"]).reshape(N, N)
        ctx = pkg.Context(N, M, K, J, case["h"])
        ctx.set_weights(cplx_arr(case["a"]).reshape(K, N), cplx_arr(case["b"]).reshape(K, M),
                        cplx_arr(case["w"]).reshape(K, N, M))
        cfgs = np.stack([cfg_words(c["cfg"], N) for c in case["configs"]])
        phi, th, E, O = ctx.evaluate(cfgs)
        orc = Oracle(N, M, K, J, case["h"])
        orc.set_weights(*ctx.get_weights())
        for t, c in enumerate(case["configs"]):
            assert rel_err(phi[t], cplx_arr(c["phi"]).reshape(K, K)) < 1e-11
            assert rel_err(E[t], cplx_arr(c["E"]).reshape(K, K)) < 1e-10
            assert rel_err(O[t][::c["O_stride"]], cplx_arr(c["O"])) < 1e-10
            ophi, oth = orc.state(cfgs[t])
            assert rel_err(th[t], oth) < 1e-11
            oE, oO = orc.local(cfgs[t])
            assert rel_err(E[t], oE) < 1e-11
            assert rel_err(O[t], oO) < 1e-11
        ctx.close()


@pytest.mark.parametrize("N,M,K,real", [(6, 12, 2, False), (8, 16, 2, True), (5, 10, 1, False), (4, 8, 3, False),
                                        (8, 16, 4, True), (66, 66, 2, True)])
def test_sr_step_parity(pkg, N, M, K, real):
    # Shapes keep 2^N well above K: when two rows of a chain land on the same
    # configuration through different flip histories, det Phi is rounding
    # noise and the reference's accept decisions depend on the last bit of its
    # own arithmetic, which no independent implementation reproduces.
    ctx, orc = make_pair(pkg, N, M, K, 0.595, 0.1 if N < 20 else 0.02, 7 + N + K, real)
    chains, m, burn = 6, 12, 5
    if N > 20:
        chains, m, burn = 3, 4, 2
    args = (9000 + N, chains, m, burn, 0.1, 2.0, 1e-9, 1000)
    e_g, info = ctx.sr_step(*args)
    e_o, oinfo = orc.sr_step(*args)
    ns = chains * m
    sg, elg, Eg = ctx.get_samples()
    so, elo, Eo = orc.samples(ns)
    assert np.array_equal(sg, so), "sampled configurations differ"
    assert info["accepted"] == oinfo["accepted"]
    assert rel_err(Eg, Eo) < 1e-11
    assert rel_err(e_g, e_o) < 1e-11
    og, sk_g, fg = ctx.get_moments()
    oo, sk_o, fo = orc.moments()
    assert rel_err(og, oo) < 1e-11
    assert rel_err(sk_g, sk_o) < 1e-10
    assert rel_err(fg, fo) < 1e-10
    # O rows (stored by the GPU) against the oracle's determinant form
    for s in [0, ns // 2, ns - 1]:
        assert rel_err(ctx.get_O(s, 1)[0], orc.sample_deriv(s)) < 1e-11
    # S·v on a random vector
    rng = np.random.default_rng(1)
    v = rng.normal(size=ctx.P) + (0 if real else 1j) * rng.normal(size=ctx.P)
    assert rel_err(ctx.apply_S(v), orc.apply_S(v)) < 1e-11
    # Solver: both stop on the reference's criteria; the GPU solution meets the
    # MINRES-QLP relative-residual bound when checked with the oracle's S.
    # Iteration counts: equal or one apart where S is well sampled (72 samples
    # for P < 2000 parameters; measured 0 or 1 apart); with 12 samples for
    # ~9000 parameters S is the regulariser plus a rank-12 term and the count
    # follows the operators' 1e-12 differences further (measured 421 vs 440).
    assert info["minres_flag"] == int(oinfo["flag"])
    it_g, it_o = int(info["minres_iters"]), int(oinfo["iters"])
    small = ctx.P < 2000
    assert abs(it_g - it_o) <= (1 if small else it_o // 10), (it_g, it_o)
    x = ctx.get_solution()
    r = np.linalg.norm(orc.apply_S(x) - fo)
    assert r <= 10 * 1e-9 * (info["anorm"] * np.linalg.norm(x) + np.linalg.norm(fo)), r
    # updated weights: both solves stop at rtol 1e-9 (measured <= 6.6e-8 and 5.0e-7)
    ag, bg, wg = ctx.get_weights()
    ao, bo, wo = orc.get_weights()
    assert rel_err(np.concatenate([ag.ravel(), bg.ravel(), wg.ravel()]),
                   np.concatenate([ao.ravel(), bo.ravel(), wo.ravel()])) < (1e-6 if small else 5e-6)
    ctx.close()


def test_consecutive_steps_and_reproducibility(pkg):
    """Three SR steps reuse one CUDA graph; a second context reproduces them bit for bit."""
    N, M, K = 8, 16, 2
    outs = []
    for rep in range(2):
        ctx, orc = make_pair(pkg, N, M, K, 0.595, 0.05, 3, True)
        es = []
        for it in range(3):
            e, info = ctx.sr_step(100 + it * 16, 16, 20, 8, 0.1, 5.0 * 0.9 ** it, 1e-9, 2000)
            es.append(e)
            if rep == 0:
                eo, _ = orc.sr_step(100 + it * 16, 16, 20, 8, 0.1, 5.0 * 0.9 ** it, 1e-9, 2000)
                assert rel_err(e, eo) < 1e-7  # weights differ at the rtol scale after step 1
        outs.append((np.array(es), ctx.get_weights()))
        ctx.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    for x, y in zip(outs[0][1], outs[1][1]):
        assert np.array_equal(x, y)


def test_nonfinite_weights_report_error(pkg):
    N, M, K = 4, 8, 2
    ctx = pkg.Context(N, M, K, synthetic_j(N), 1.0)
    a, b, w = helpers.random_weights(N, M, K, 0.1, 1, real=True)
    w[0, 0, 0] = np.nan
    ctx.set_weights(a, b, w)
    with pytest.raises(pkg.NqesError) as e:
        ctx.sr_step(1, 4, 4, 2, 0.1, 1.0, 1e-9, 100)
    assert e.value.status == pkg.ERR_NONFINITE
    ctx.close()


def test_training_reaches_exact_diagonalisation(pkg):
    """N=8, K=2, h=1: SR training (lambda 40 -> 5, lr 0.1) brings the two lowest
    energies per site to exact diagonalisation within the variational error of
    an M=2N RBM (1% of |E|), averaged over the last 10 steps."""
    with open(os.path.join(GOLDEN, "ed_golden.json")) as f:
        ed = [c for c in json.load(f)["cases"] if c["N"] == 8 and c["h"] == 1.0][0]
    want = np.array(ed["evals_per_site"][:2])
    N, M, K = 8, 16, 2
    ctx = pkg.Context(N, M, K, synthetic_j(N), ed["h"])
    ctx.set_weights(*helpers.random_weights(N, M, K, 0.05, 11, real=True))
    lr, reglam, hist = 0.1, 40.0, []
    chains, m = 256, 200
    for it in range(150):
        e, info = ctx.sr_step(5000 + it * chains, chains, m, 32, max(lr, 0.01), max(reglam, 5.0), 1e-9, 5000)
        lr *= 0.99
        reglam *= 0.9
        hist.append(np.sort(np.linalg.eigvals(e / N).real))
    final = np.mean(hist[-10:], axis=0)
    print("final", final, "ED", want)
    assert np.all(final >= want - 2e-3), (final, want)          # variational (up to noise)
    assert np.all(np.abs(final - want) < 0.01 * np.abs(want)), (final, want)
    ctx.close()


@pytest.mark.parametrize("N,M,K,real", [(6, 12, 2, False), (8, 16, 2, True), (5, 10, 3, False)])
def test_correlations_match_oracle(pkg, N, M, K, real):
    """x, z, xx, zz from one correlation pass (code/rbm.cc:730-826): same chains
    as the reference's four passes with one seed, results within 1e-10."""
    ctx, orc = make_pair(pkg, N, M, K, 0.8, 0.15, 40 + N, real)
    rng = np.random.default_rng(N)
    V = rng.normal(size=(K, K)) + 1j * rng.normal(size=(K, K))
    got = ctx.correlations(77, 6, 15, 5, V)
    want = orc.correlations(77, 6, 15, 5, V)
    for g, w in zip(got, want):
        assert np.max(np.abs(g - w)) <= 1e-10 * max(1.0, np.max(np.abs(w)))
    ctx.close()


@pytest.mark.parametrize("N,M,K,chains,m", [(8, 16, 2, 16, 30), (32, 64, 2, 32, 20), (12, 24, 3, 8, 20),
                                            (20, 40, 1, 8, 10), (64, 128, 4, 4, 6), (10, 300, 4, 4, 6),
                                            (19, 19, 3, 8, 10), (72, 144, 4, 4, 6), (68, 136, 3, 4, 6),
                                            (86, 172, 1, 8, 6), (96, 192, 4, 4, 6)])
def test_mixed_precision_keeps_fp64_chains(pkg, N, M, K, chains, m):
    """MIXED: FP32 decisions with a certified bound and an exact FP64 fallback
    give the FP64 chains bit for bit (decision-warp form for up to 32 hidden
    units per lane, block form beyond: M=300, K=4; the serving loop's shapes:
    M = N odd, 32 units per lane at K = 3, 4, N > 64 up to N96 M192 K4, the
    largest request it serves); energies within 1e-6 relative, FP32
    log-derivatives, moments and S·v (factored FP32 passes) within 1e-5 / 1e-4,
    the updated weights within 5e-5 (2e-4 where 24 samples meet P > 10^4)."""
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.05 if N < 20 else 0.02, 5 + N, real=True)
    out = {}
    P = K * (N + M + N * M)
    vrand = np.random.default_rng(N + M).normal(size=P).astype(np.complex128)
    for prec in (pkg.PRECISION_FP64, pkg.PRECISION_MIXED):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_PRECISION, prec)
        e, info = ctx.sr_step(4242, chains, m, 10, 0.1, 5.0, 1e-9, 2000)
        spins, eloc, E = ctx.get_samples()
        out[prec] = dict(e=e, info=info, spins=spins, E=E, O=ctx.get_O(0, 4), acc=ctx.get_accepts(),
                         mom=ctx.get_moments(), w=np.concatenate([x.ravel() for x in ctx.get_weights()]),
                         sv=ctx.apply_S(vrand), Oall=ctx.get_O(0, chains * m))
        ctx.close()
    f, x = out[0], out[1]
    assert np.array_equal(f["spins"], x["spins"]), "mixed chains left the FP64 chains"
    assert np.array_equal(f["acc"], x["acc"])
    assert x["info"]["precision"] == 1
    assert rel_err(x["E"], f["E"]) < 1e-5
    assert rel_err(x["e"], f["e"]) < 1e-6
    assert rel_err(x["O"], f["O"]) < 1e-5
    assert rel_err(x["Oall"], f["Oall"]) < 1e-5
    # o, the regularised diagonal of S and the force, from the factored passes
    for a, b in zip(x["mom"], f["mom"]):
        assert rel_err(a, b) < 1e-4
    # the factored S·v (FP32 passes) against the dense FP64 one on the same chains
    assert rel_err(x["sv"], f["sv"]) < 1e-4
    # the update solves S x = f with FP32 operator passes; with 24 samples for
    # P > 10^4 parameters S is the regulariser plus a rank-24 term, and the
    # solve amplifies the operator's ~1e-6 rounding differences
    assert rel_err(x["w"], f["w"]) < (5e-5 if P < 10000 else 2e-4)


@pytest.mark.parametrize("N,M,K,chains,m", [(8, 16, 2, 16, 30), (32, 64, 2, 24, 20), (12, 24, 3, 8, 20),
                                            (16, 300, 4, 4, 6), (20, 40, 1, 8, 10)])
def test_reject_filter_is_bit_identical(pkg, N, M, K, chains, m):
    """The FP32 rejection filter only skips FP64 work of proposals it proves
    rejected: configurations, accept counts, E, O, moments, e_mat and the
    updated weights are bit-identical with the filter on and off."""
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.05 if N < 20 else 0.02, 3 + N, real=True)
    out = []
    for filt in (0, 1):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_REJECT_FILTER, filt)
        e, info = ctx.sr_step(777, chains, m, 6, 0.1, 5.0, 1e-9, 2000)
        spins, eloc, E = ctx.get_samples()
        out.append(dict(e=e, spins=spins, E=E, O=ctx.get_O(0, chains * m), acc=ctx.get_accepts(),
                        mom=ctx.get_moments(), w=np.concatenate([x.ravel() for x in ctx.get_weights()])))
        ctx.close()
    for key in out[0]:
        for a, b in zip(out[0][key] if isinstance(out[0][key], tuple) else [out[0][key]],
                        out[1][key] if isinstance(out[1][key], tuple) else [out[1][key]]):
            assert np.array_equal(a, b), key


@pytest.mark.parametrize("N,M,K,chains,m", [(8, 16, 2, 16, 30), (12, 24, 3, 8, 20)])
def test_mixed_exact_path_keeps_fp64_chains(pkg, N, M, K, chains, m):
    """MIXED with every accept decision taken by its exact FP64 path follows
    the FP64 chains."""
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.05, 5 + N, real=True)
    spins = []
    for prec in (pkg.PRECISION_FP64, pkg.PRECISION_MIXED):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_PRECISION, prec)
        ctx.set_option(pkg.OPT_MIXED_EXACT, 1)
        e, info = ctx.sr_step(4242, chains, m, 10, 0.1, 5.0, 1e-9, 2000)
        spins.append(ctx.get_samples()[0])
        if prec == pkg.PRECISION_MIXED:
            assert info["exact_decisions"] > 0
        ctx.close()
    assert np.array_equal(spins[0], spins[1])


@pytest.mark.parametrize("N,M,K,chains,m", [(8, 16, 2, 16, 30), (32, 64, 2, 32, 20), (12, 24, 3, 8, 20),
                                            (20, 40, 1, 8, 10), (64, 128, 4, 4, 6), (70, 45, 3, 8, 10),
                                            (100, 200, 2, 4, 8), (10, 300, 4, 4, 6)])
def test_tensor_core_rows_pass_matches_cuda_cores(pkg, N, M, K, chains, m):
    """MIXED: the tcgen05 rows and column passes (BF16 x3 splits, FP32
    accumulation) and the FP32 CUDA-core passes give the same S·v and moments
    to FP32 rounding, the same chains
    and energies, and updated weights within the solve's FP32 sensitivity
    (forced on wherever the shape fits: K = 1..4, N > 64, M not a multiple of
    16; M = 300 exceeds the tensor-core shape and checks that the option
    changes nothing there)."""
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.05 if N < 20 else 0.02, 11 + N, real=True)
    P = K * (N + M + N * M)
    vrand = np.random.default_rng(3 * N + M).normal(size=P).astype(np.complex128)
    out = []
    for tc in (0, 1):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_PRECISION, pkg.PRECISION_MIXED)
        ctx.set_option(pkg.OPT_TENSOR_CORES, 2 * tc)
        e, info = ctx.sr_step(99, chains, m, 10, 0.1, 5.0, 1e-9, 2000)
        out.append(dict(e=e, spins=ctx.get_samples()[0], sv=ctx.apply_S(vrand), mom=ctx.get_moments(),
                        w=np.concatenate([x.ravel() for x in ctx.get_weights()])))
        ctx.close()
    a, b = out
    assert np.array_equal(a["spins"], b["spins"])
    assert rel_err(b["sv"], a["sv"]) < 1e-5
    for x, y in zip(b["mom"], a["mom"]):  # o, lambda-scaled diagonal of S, force
        assert rel_err(x, y) < 1e-5
    assert rel_err(b["e"], a["e"]) < 1e-6
    assert rel_err(b["w"], a["w"]) < (5e-5 if P < 10000 else 2e-4)


@pytest.mark.parametrize("N,M,K,chains,m", [(8, 16, 2, 16, 30), (32, 64, 2, 32, 20), (12, 24, 3, 8, 20),
                                            (20, 40, 1, 8, 10), (64, 128, 4, 4, 6), (66, 66, 2, 4, 8),
                                            (10, 300, 4, 4, 6)])
def test_certified_matches_fp64(pkg, N, M, K, chains, m):
    """CERTIFIED: the mixed form's sampler (certified FP32 decisions, exact FP64
    fallback) with FP64 outputs gives the FP64 form's configurations and accept
    counts bit for bit, and its local energies, log-derivatives, moments and
    S·v to FP64 rounding (tanh of the exact theta instead of the FP64 sampler's
    incrementally updated tanh); M = 300 runs the FP64 sampler (beyond the
    decision-warp shapes)."""
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.05 if N < 20 else 0.02, 7 + N, real=True)
    P = K * (N + M + N * M)
    vrand = np.random.default_rng(N + 2 * M).normal(size=P).astype(np.complex128)
    out = {}
    for prec in (pkg.PRECISION_FP64, pkg.PRECISION_CERTIFIED):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_PRECISION, prec)
        e, info = ctx.sr_step(4243, chains, m, 10, 0.1, 5.0, 1e-9, 2000)
        spins, eloc, E = ctx.get_samples()
        out[prec] = dict(e=e, info=info, spins=spins, E=E, O=ctx.get_O(0, chains * m), acc=ctx.get_accepts(),
                         mom=ctx.get_moments(), sv=ctx.apply_S(vrand),
                         w=np.concatenate([x.ravel() for x in ctx.get_weights()]))
        ctx.close()
    f, c = out[pkg.PRECISION_FP64], out[pkg.PRECISION_CERTIFIED]
    assert np.array_equal(f["spins"], c["spins"]), "certified chains left the FP64 chains"
    assert np.array_equal(f["acc"], c["acc"])
    assert c["info"]["precision"] == pkg.PRECISION_CERTIFIED
    assert rel_err(c["E"], f["E"]) < 1e-11
    assert rel_err(c["O"], f["O"]) < 1e-11
    assert rel_err(c["e"], f["e"]) < 1e-11
    for a, b in zip(c["mom"], f["mom"]):
        assert rel_err(a, b) < 1e-10
    assert rel_err(c["sv"], f["sv"]) < 1e-10
    # the update: MINRES-QLP stops at rtol 1e-9, so two solves whose operators
    # differ by rounding (1e-13 here) agree to the solver's tolerance times the
    # conditioning of S, not to rounding; with 24 samples for P > 10^4
    # parameters S is the regulariser plus a rank-24 term
    assert rel_err(c["w"], f["w"]) < (1e-6 if P < 10000 else 5e-6)


# P = 304, 4288, 4288, 816 and then one shape per wider thread layout of the
# fused kernel: P = 3200 (5 columns x 640 threads), 3248 (7 x 480), 6640 (17 x 416)
@pytest.mark.parametrize("N,M,K,prec", [(8, 16, 2, 0), (32, 64, 2, 0), (32, 64, 2, 2), (12, 20, 3, 0),
                                        (32, 96, 1, 2), (24, 64, 2, 2), (40, 80, 2, 2)])
def test_fused_sv_matches_two_pass(pkg, N, M, K, prec):
    """The fused S·v (one read of the FP64 O per product, double-float
    arithmetic on the FP32 pipe) against the two FP64 passes on the same
    samples: S·v within 1e-13 relative, and a whole SR step (MINRES-QLP
    iterations, flag, e_mat, updated weights) agreeing to the solver's
    rounding."""
    out = {}
    for fused in (0, 1):
        ctx = pkg.Context(N, M, K, synthetic_j(N), 0.595)
        ctx.set_weights(*pkg.synthetic_weights(N, M, K, 0.02, 3))
        ctx.set_option(pkg.OPT_PRECISION, prec)
        ctx.set_option(pkg.OPT_FUSED_SV, fused)
        e, info = ctx.sr_step(71, 64, 50, 16, 0.1, 10.0, 1e-9, 100000)
        rng = np.random.default_rng(9)
        vs = [rng.normal(size=ctx.P) for _ in range(3)]
        out[fused] = dict(e=e, info=info, sv=[ctx.apply_S(v) for v in vs], w=ctx.get_weights(),
                          spins=ctx.get_samples()[0])
        ctx.close()
    a, b = out[0], out[1]
    assert np.array_equal(a["spins"], b["spins"])
    for x, y in zip(a["sv"], b["sv"]):
        assert rel_err(y, x) < 1e-13, rel_err(y, x)
    assert a["info"]["minres_flag"] == b["info"]["minres_flag"]
    it_a, it_b = int(a["info"]["minres_iters"]), int(b["info"]["minres_iters"])
    assert abs(it_a - it_b) <= max(2, it_a // 20), (it_a, it_b)  # Krylov counts move with the last bits
    assert rel_err(b["e"], a["e"]) < 1e-13
    wa = np.concatenate([z.ravel() for z in a["w"]])
    wb = np.concatenate([z.ravel() for z in b["w"]])
    assert rel_err(wb, wa) < 1e-6  # the solves agree to the rtol scale


@pytest.mark.parametrize("mode", [2, 1])
def test_mixed_energies_along_the_fp64_trajectory(pkg, mode):
    """The mixed form's energy error beyond the first step, at the plain
    configuration N8 M16 K2 (128 chains x 200 samples, burn-in 64, the
    reference schedule lambda 40 -> 1, lr 0.1 -> 0.01): before every step the
    mixed context takes the FP64 context's weights, so both sample the same
    Markov chains and the difference is the arithmetic alone. Max over 40
    steps of the per-site energies' relative difference: <= 1e-6 (the stated
    target) with the default energies (NQES_OPT_MIXED_ENERGY64 = 2: tanh from
    FP32, double-float ratio products), <= 1e-10 with tanh in FP64 (1)."""
    N, M, K, chains = 8, 16, 2, 128
    J = synthetic_j(N)
    f = pkg.Context(N, M, K, J, 0.595)
    x = pkg.Context(N, M, K, J, 0.595)
    f.set_weights(*pkg.synthetic_weights(N, M, K, 0.01, 20240601))
    x.set_option(pkg.OPT_PRECISION, pkg.PRECISION_MIXED)
    x.set_option(pkg.OPT_MIXED_ENERGY64, mode)
    worst = 0.0
    for t in range(40):
        lr, lam = max(0.1 * 0.99 ** t, 0.01), max(40.0 * 0.9 ** t, 1.0)
        x.set_weights(*f.get_weights())
        args = (777 + t * chains, chains, 200, 64, lr, lam, 1e-9, 100000)
        ef, _ = f.sr_step(*args)
        em, _ = x.sr_step(*args)
        assert np.array_equal(f.get_samples()[0], x.get_samples()[0])
        vf, vm = (np.sort(np.linalg.eigvals(e / N).real) for e in (ef, em))
        worst = max(worst, float(np.max(np.abs(vm - vf) / np.abs(vf))))
    print(f"energy mode {mode}: max relative energy difference over 40 steps:", worst)
    assert worst <= (1e-6 if mode == 2 else 1e-10)
    f.close()
    x.close()


@pytest.mark.parametrize("N,M,K,prec", [(32, 64, 2, 1), (32, 64, 2, 2), (12, 24, 3, 1), (20, 40, 1, 2)])
def test_sampler_plan_does_not_change_results(pkg, N, M, K, prec):
    """NQES_OPT_SAMPLER_PLAN: one, two, four or eight warps per chain, tables
    staged or read from global memory, give the same bits (configurations,
    local energies, e_mat, updated weights): the helper warps form the samples
    in a fixed order whatever their number."""
    J = synthetic_j(N)
    w = helpers.random_weights(N, M, K, 0.02, 17 + N, real=True)
    ref = None
    for plan in (0, 1, 2, 4, 8, 17, 18, 20, 24):
        ctx = pkg.Context(N, M, K, J, 0.595)
        ctx.set_weights(*w)
        ctx.set_option(pkg.OPT_PRECISION, prec)
        ctx.set_option(pkg.OPT_SAMPLER_PLAN, plan)
        e, info = ctx.sr_step(321, 24, 10, 6, 0.1, 5.0, 1e-9, 2000)
        spins, eloc, E = ctx.get_samples()
        got = dict(e=e, spins=spins, E=E, w=np.concatenate([x.ravel() for x in ctx.get_weights()]),
                   it=info["minres_iters"])
        ctx.close()
        if ref is None:
            ref = got
            continue
        assert np.array_equal(got["spins"], ref["spins"]), plan
        assert np.array_equal(got["E"], ref["E"]), plan
        assert np.array_equal(got["e"], ref["e"]), plan
        assert got["it"] == ref["it"], plan
        assert np.array_equal(got["w"], ref["w"]), plan
