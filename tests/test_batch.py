"""Batched multi-solve (one CUDA graph launch per SR step for several solves)
and the launch-shape autotuner."""
import numpy as np
import pytest

import __graft_entry__ as ge
import helpers
from helpers import synthetic_j

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


# (N, M, K, h, J exponent, precision, real weights)
MEMBERS = [(8, 16, 2, 0.5, 1.2, 0, True), (12, 24, 3, 1.0, 0.9, 1, True), (10, 20, 1, 0.8, 1.5, 0, False),
           (16, 32, 2, 0.3, 1.1, 1, True)]


def make(pkg, idx, spec):
    N, M, K, h, alpha, prec, real = spec
    ctx = pkg.Context(N, M, K, synthetic_j(N, alpha), h)
    ctx.set_weights(*helpers.random_weights(N, M, K, 0.05, 100 + idx, real=real))
    ctx.set_option(pkg.OPT_PRECISION, prec)
    return ctx


def step_args(t, n):
    seeds = [1000 + 97 * i + t * 64 for i in range(n)]
    chains = [8 + 4 * i for i in range(n)]
    m = [10 + i for i in range(n)]
    burn = [4] * n
    lr = [0.1] * n
    reglam = [5.0 * 0.9 ** t] * n
    return seeds, chains, m, burn, lr, reglam, [1e-9] * n, [2000] * n


def test_batch_equals_individual_steps(pkg):
    """Each member's e_mat, samples and updated weights are those of nqes_sr_step
    on the same context, bit for bit, over consecutive batched steps."""
    alone = [make(pkg, i, s) for i, s in enumerate(MEMBERS)]
    mixed = [make(pkg, i, s) for i, s in enumerate(MEMBERS)]
    batch = pkg.Batch(mixed)
    n = len(MEMBERS)
    for t in range(2):
        seeds, chains, m, burn, lr, reglam, rtol, maxit = step_args(t, n)
        emats, infos, stats, ms = batch.sr_step(seeds, chains, m, burn, lr, reglam, rtol, maxit)
        assert stats == [0] * n and ms > 0
        for i, c in enumerate(alone):
            e, info = c.sr_step(seeds[i], chains[i], m[i], burn[i], lr[i], reglam[i], rtol[i], maxit[i])
            assert np.array_equal(e, emats[i]), (t, i)
            assert info["minres_iters"] == infos[i]["minres_iters"]
            assert info["accepted"] == infos[i]["accepted"]
            assert np.array_equal(c.get_samples()[0], mixed[i].get_samples()[0])
            for x, y in zip(c.get_weights(), mixed[i].get_weights()):
                assert np.array_equal(x, y)
    batch.close()
    for c in alone + mixed:
        c.close()


# grouped loop body: three MIXED members of one S·v kernel variant, a MIXED
# member of another, one whose rows pass runs on the tensor cores (N M = 4096:
# its own launches), a CERTIFIED member (fused FP64 S·v: its own launches)
GROUPED = [(16, 32, 2, 0.5, 1.2, 1, True), (16, 32, 2, 0.9, 1.0, 1, True), (16, 32, 2, 0.7, 1.4, 1, True),
           (20, 40, 3, 0.6, 1.1, 1, True), (64, 64, 2, 0.8, 1.2, 1, True), (12, 24, 2, 0.4, 1.3, 2, True)]


def test_grouped_loop_body_equals_individual_steps(pkg):
    """The batch's loop body launches each MINRES-QLP kernel once for all its
    members (grouped by S·v kernel variant; members without a grouped S·v run
    it on their own streams): every member's e_mat, iterations, samples and
    updated weights equal nqes_sr_step on it, bit for bit, over two steps."""
    alone = [make(pkg, i, s) for i, s in enumerate(GROUPED)]
    mixed = [make(pkg, i, s) for i, s in enumerate(GROUPED)]
    batch = pkg.Batch(mixed)
    n = len(GROUPED)
    for t in range(2):
        seeds, chains, m, burn, lr, reglam, rtol, maxit = step_args(t, n)
        emats, infos, stats, ms = batch.sr_step(seeds, chains, m, burn, lr, reglam, rtol, maxit)
        assert stats == [0] * n and ms > 0
        for i, c in enumerate(alone):
            e, info = c.sr_step(seeds[i], chains[i], m[i], burn[i], lr[i], reglam[i], rtol[i], maxit[i])
            assert np.array_equal(e, emats[i]), (t, i)
            assert info["minres_iters"] == infos[i]["minres_iters"], (t, i)
            assert np.array_equal(c.get_samples()[0], mixed[i].get_samples()[0])
            for x, y in zip(c.get_weights(), mixed[i].get_weights()):
                assert np.array_equal(x, y), (t, i)
    batch.close()
    for c in alone + mixed:
        c.close()


def test_tensor_core_members_equal_individual_steps(pkg):
    """Members with both factored passes on the tensor cores
    (NQES_OPT_TENSOR_CORES 2: their rows and column passes run as their own
    launches inside the grouped loop body) beside a member in the grouped
    CUDA-core passes: each equals nqes_sr_step on it, bit for bit."""
    spec = [(16, 32, 2, 0.6, 1.2, 1, True), (20, 40, 3, 0.8, 1.0, 1, True), (16, 32, 2, 0.7, 1.3, 1, True)]
    tcs = [2, 2, 1]
    alone = [make(pkg, i, s) for i, s in enumerate(spec)]
    mixed = [make(pkg, i, s) for i, s in enumerate(spec)]
    for c, d, tc in zip(alone, mixed, tcs):
        c.set_option(pkg.OPT_TENSOR_CORES, tc)
        d.set_option(pkg.OPT_TENSOR_CORES, tc)
    batch = pkg.Batch(mixed)
    n = len(spec)
    for t in range(2):
        seeds, chains, m, burn, lr, reglam, rtol, maxit = step_args(t, n)
        emats, infos, stats, _ = batch.sr_step(seeds, chains, m, burn, lr, reglam, rtol, maxit)
        assert stats == [0] * n
        for i, c in enumerate(alone):
            e, info = c.sr_step(seeds[i], chains[i], m[i], burn[i], lr[i], reglam[i], rtol[i], maxit[i])
            assert np.array_equal(e, emats[i]), (t, i)
            assert info["minres_iters"] == infos[i]["minres_iters"], (t, i)
            for x, y in zip(c.get_weights(), mixed[i].get_weights()):
                assert np.array_equal(x, y), (t, i)
    batch.close()
    for c in alone + mixed:
        c.close()


def test_large_rows_group_equals_individual_steps(pkg):
    """A rows group of the loop body with more than six waves of blocks runs
    the rows pass with four rows a thread group (half the blocks of the
    one-solve form, the same arithmetic per row): five MIXED members of
    N20 M40 K2 at 128 chains x 100 samples give each member's e_mat,
    iterations and updated weights of nqes_sr_step on it, bit for bit."""
    spec = [(20, 40, 2, 0.5 + 0.1 * i, 1.2, 1, True) for i in range(5)]
    alone = [make(pkg, i, s) for i, s in enumerate(spec)]
    mixed = [make(pkg, i, s) for i, s in enumerate(spec)]
    batch = pkg.Batch(mixed)
    n = len(spec)
    seeds = [500 + 1000 * i for i in range(n)]
    args = (seeds, [128] * n, [100] * n, [8] * n, [0.1] * n, [5.0] * n, [1e-9] * n, [2000] * n)
    emats, infos, stats, _ = batch.sr_step(*args)
    assert stats == [0] * n
    for i, c in enumerate(alone):
        e, info = c.sr_step(*[a[i] for a in args])
        assert np.array_equal(e, emats[i]), i
        assert info["minres_iters"] == infos[i]["minres_iters"], i
        for x, y in zip(c.get_weights(), mixed[i].get_weights()):
            assert np.array_equal(x, y), i
    batch.close()
    for c in alone + mixed:
        c.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_autotune_keeps_the_chains(pkg, prec):
    """The autotuner only changes launch shapes: the chains are the same and
    energies agree to FP64 rounding of the reduction order."""
    N, M, K = 16, 32, 2
    out = []
    for tune in (0, 1):
        c = pkg.Context(N, M, K, synthetic_j(N), 0.6)
        c.set_weights(*helpers.random_weights(N, M, K, 0.05, 3, real=True))
        c.set_option(pkg.OPT_PRECISION, prec)
        c.set_option(pkg.OPT_AUTOTUNE, tune)
        es = []
        for t in range(2):
            e, _ = c.sr_step(50 + t * 32, 32, 20, 5, 0.1, 5.0, 1e-9, 2000)
            es.append(e)
        out.append((es, c.get_samples()[0]))
        c.close()
    assert np.array_equal(out[0][1], out[1][1])
    for a, b in zip(out[0][0], out[1][0]):
        assert np.max(np.abs(a - b)) <= 1e-9 * np.max(np.abs(b))


def test_batch_rebuilds_after_a_member_changes_its_hamiltonian(pkg):
    """A member switched to the Heisenberg-like local energy between batched
    steps gets that energy in the next batched step (the batch graph is
    rebuilt), equal to stepping a context set up that way alone."""
    from test_oracle_heisenberg import xxz_j
    N, M, K = 8, 16, 2
    w = helpers.random_weights(N, M, K, 0.05, 7, real=True)
    member = pkg.Context(N, M, K, xxz_j(N), 0.0)
    member.set_weights(*w)
    batch = pkg.Batch([member])
    args = ([31], [8], [10], [4], [0.1], [5.0], [1e-9], [2000])
    batch.sr_step(*args)  # ising-like form with the xxz couplings
    member.set_weights(*w)
    member.set_hamiltonian(pkg.HAM_HEISENBERG_LIKE, -1.0)
    emats, _, stats, _ = batch.sr_step(*args)
    assert stats == [0]
    alone = pkg.Context(N, M, K, xxz_j(N), 0.0)
    alone.set_weights(*w)
    alone.set_hamiltonian(pkg.HAM_HEISENBERG_LIKE, -1.0)
    e, _ = alone.sr_step(31, 8, 10, 4, 0.1, 5.0, 1e-9, 2000)
    assert np.array_equal(e, emats[0])
    batch.close()
    member.close()
    alone.close()


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_after_a_member_reallocates_its_buffers(pkg, prec):
    """A solo step at another chain count (or a precision switch with a solo
    step in between) frees and reallocates a member's step buffers; the next
    batched step at the original shape must not replay a graph that points at
    the freed memory. Its results equal a fresh context's through the same
    steps."""
    N, M, K = 8, 16, 2
    w = helpers.random_weights(N, M, K, 0.05, 21, real=True)

    def fresh():
        c = pkg.Context(N, M, K, synthetic_j(N), 0.7)
        c.set_weights(*w)
        c.set_option(pkg.OPT_PRECISION, prec)
        return c

    member, ref = fresh(), fresh()
    batch = pkg.Batch([member])
    args = lambda t: ([40 + 16 * t], [16], [12], [4], [0.1], [5.0], [1e-9], [2000])
    e_b, _, stats, _ = batch.sr_step(*args(0))
    e_r, _ = ref.sr_step(40, 16, 12, 4, 0.1, 5.0, 1e-9, 2000)
    assert stats == [0] and np.array_equal(e_b[0], e_r)
    # solo step at another chain count: new buffers; then (prec 1) a solo step
    # in the other precision and back, which reallocates them once more
    for c in (member, ref):
        c.sr_step(99, 24, 12, 4, 0.1, 5.0, 1e-9, 2000)
        if prec:
            c.set_option(pkg.OPT_PRECISION, 0)
            c.sr_step(101, 16, 12, 4, 0.1, 5.0, 1e-9, 2000)
            c.set_option(pkg.OPT_PRECISION, prec)
    e_b, _, stats, _ = batch.sr_step(*args(1))
    e_r, _ = ref.sr_step(56, 16, 12, 4, 0.1, 5.0, 1e-9, 2000)
    assert stats == [0] and np.array_equal(e_b[0], e_r)
    assert np.array_equal(member.get_samples()[0], ref.get_samples()[0])
    for x, y in zip(member.get_weights(), ref.get_weights()):
        assert np.array_equal(x, y)
    batch.close()
    member.close()
    ref.close()
