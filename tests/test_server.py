"""Serving loop: admission by device footprint, continuous batching in lanes
by size class, results independent of what else runs."""
import numpy as np
import pytest

import __graft_entry__ as ge
import helpers
from helpers import synthetic_j


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


def test_footprint_counts_the_o_matrix(pkg):
    """The footprint bound grows with the samples and covers O (FP64 real,
    FP64 complex) or, in the mixed form, its factors (K^2 (M + 1) floats per
    sample)."""
    N, M, K, c, m = 32, 64, 2, 128, 200
    P = K * (N + M + N * M)
    f64 = pkg.footprint_bytes(N, M, K, c, m, pkg.PRECISION_FP64)
    c128 = pkg.footprint_bytes(N, M, K, c, m, pkg.PRECISION_FP64, complex_arith=True)
    mix = pkg.footprint_bytes(N, M, K, c, m, pkg.PRECISION_MIXED)
    assert f64 >= c * m * P * 8 and c128 >= c * m * P * 16 and mix >= c * m * K * K * (M + 1) * 4
    assert mix < f64 < c128
    assert pkg.footprint_bytes(N, M, K, c, 2 * m) > f64


def test_server_reports_failures_without_hanging(pkg):
    """Host logic: a request that can never fit fails with NQES_ERR_OOM; on a
    machine without a GPU an admitted request fails with NQES_ERR_CUDA."""
    torch = pytest.importorskip("torch")
    srv = pkg.Server(hbm_budget_bytes=1 << 20, max_active=2)
    big = srv.submit(32, 64, 2, synthetic_j(32), chains=128, samples_per_chain=200)
    res = srv.wait_all(1, timeout=30)
    srv.close()
    assert [r["id"] for r in res] == [big] and res[0]["status"] == pkg.ERR_OOM
    if not torch.cuda.is_available():
        srv = pkg.Server(hbm_budget_bytes=1 << 40, max_active=2)
        srv.submit(8, 16, 2, synthetic_j(8), max_steps=2)
        res = srv.wait_all(1, timeout=30)
        srv.close()
        assert len(res) == 1 and res[0]["status"] == pkg.ERR_CUDA


SPECS = [dict(n=8, m=16, k=2, h=0.7, prec=0, seed=11), dict(n=12, m=12, k=3, h=1.1, prec=1, seed=23),
         dict(n=10, m=20, k=1, h=0.4, prec=0, seed=37), dict(n=16, m=32, k=2, h=0.9, prec=1, seed=41)]


def submit_all(pkg, srv, specs):
    ids = []
    for s in specs:
        w = helpers.random_weights(s["n"], s["m"], s["k"], 0.05, s["seed"], real=True)
        ids.append(srv.submit(s["n"], s["m"], s["k"], synthetic_j(s["n"]), weights=w, h=s["h"], seed=s["seed"],
                              chains=16, samples_per_chain=20, burn_in=5, reglam0=5.0, tol=1e-12, max_steps=4,
                              precision=s["prec"]))
    return ids


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix(pkg):
    """Each solve's energies are bit-identical whether it runs alone or batched
    with solves of other shapes and precisions."""
    alone = {}
    for s in SPECS:
        srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=1)
        (rid,) = submit_all(pkg, srv, [s])
        (r,) = srv.wait_all(1)
        srv.close()
        assert r["status"] == 0 and r["steps"] == 4
        alone[s["seed"]] = r
    srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=8)
    ids = submit_all(pkg, srv, SPECS)
    res = {r["id"]: r for r in srv.wait_all(len(SPECS))}
    srv.close()
    for rid, s in zip(ids, SPECS):
        r, a = res[rid], alone[s["seed"]]
        assert r["status"] == 0 and r["steps"] == a["steps"]
        assert r["energies"] == a["energies"] and r["best"] == a["best"]


@pytest.mark.gpu
def test_admission_waits_for_memory(pkg):
    """With room for one solve at a time, every solve still completes; later
    ones queue until memory frees up."""
    one = max(pkg.footprint_bytes(s["n"], s["m"], s["k"], 16, 20, s["prec"]) for s in SPECS)
    srv = pkg.Server(hbm_budget_bytes=int(1.5 * one), max_active=8)
    ids = submit_all(pkg, srv, SPECS)
    res = srv.wait_all(len(SPECS))
    srv.close()
    assert sorted(r["id"] for r in res) == sorted(ids)
    assert all(r["status"] == 0 for r in res)
    assert max(r["t_queued"] for r in res) > 0.0


@pytest.mark.gpu
def test_turnover_rebuilds_the_batch(pkg):
    """One active solve at a time, one step each, alternating shapes: every
    retirement is followed by an admission whose context may reuse the retired
    one's address; each solve still gets its own batch and the results of
    running it alone."""
    specs = [dict(SPECS[i % 2], seed=101 + i) for i in range(6)]

    def run(srv, ss):
        ids = []
        for s in ss:
            w = helpers.random_weights(s["n"], s["m"], s["k"], 0.05, s["seed"], real=True)
            ids.append(srv.submit(s["n"], s["m"], s["k"], synthetic_j(s["n"]), weights=w, h=s["h"], seed=s["seed"],
                                  chains=16, samples_per_chain=20, burn_in=5, reglam0=5.0, tol=1e-12, max_steps=1,
                                  precision=s["prec"]))
        return ids, {r["id"]: r for r in srv.wait_all(len(ss))}

    srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=1)
    ids, res = run(srv, specs)
    srv.close()
    for rid, s in zip(ids, specs):
        alone = pkg.Server(hbm_budget_bytes=1 << 36, max_active=1)
        (aid,), ares = run(alone, [s])
        alone.close()
        assert res[rid]["status"] == 0 and ares[aid]["status"] == 0
        assert res[rid]["energies"] == ares[aid]["energies"]


@pytest.mark.gpu
def test_request_arriving_during_a_step_equals_running_alone(pkg):
    """A request submitted while another solve's batched steps are running on
    the device joins that batch at its next step (both are of the same size
    class, so they share a lane); both results equal those of running each
    alone, bit for bit."""
    import time
    big = dict(n=24, m=48, k=2, h=0.6, prec=1, seed=51)
    small = dict(n=12, m=24, k=2, h=0.9, prec=0, seed=53)

    def submit(srv, s, steps, chains, m):
        w = helpers.random_weights(s["n"], s["m"], s["k"], 0.05, s["seed"], real=True)
        return srv.submit(s["n"], s["m"], s["k"], synthetic_j(s["n"]), weights=w, h=s["h"], seed=s["seed"],
                          chains=chains, samples_per_chain=m, burn_in=8, reglam0=5.0, tol=1e-12, max_steps=steps,
                          precision=s["prec"])

    alone = {}
    for s, args in ((big, (12, 128, 100)), (small, (3, 16, 20))):
        srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=4)
        submit(srv, s, *args)
        (r,) = srv.wait_all(1)
        srv.close()
        assert r["status"] == 0
        alone[s["seed"]] = r
    srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=4)
    t0 = time.perf_counter()
    id_big = submit(srv, big, 12, 128, 100)
    # wait until the big solve's batched steps are under way, then submit
    deadline = time.perf_counter() + 60
    while srv.times()["steps"] < 2 and time.perf_counter() < deadline:
        time.sleep(0.001)
    t_small = time.perf_counter() - t0
    id_small = submit(srv, small, 3, 16, 20)
    res = {r["id"]: r for r in srv.wait_all(2)}
    srv.close()
    rb, rs = res[id_big], res[id_small]
    assert rb["status"] == 0 and rs["status"] == 0
    # the small solve was admitted while the big one was still stepping
    assert t_small + rs["t_queued"] < rb["t_total"], (t_small, rs["t_queued"], rb["t_total"])
    for r, s in ((rb, big), (rs, small)):
        a = alone[s["seed"]]
        assert r["steps"] == a["steps"] and r["energies"] == a["energies"] and r["best"] == a["best"]


@pytest.mark.gpu
def test_size_classes_run_side_by_side(pkg):
    """A small solve submitted after a large one (another size class) is not
    held back by the large one's steps: it finishes first, and both results
    equal running each alone."""
    big = dict(n=64, m=128, k=2, h=0.6, prec=1, seed=61)     # P = 16768: the middle lane
    small = dict(n=10, m=20, k=2, h=0.9, prec=0, seed=63)    # P = 440: the first lane

    def submit(srv, s, steps, chains, m):
        w = helpers.random_weights(s["n"], s["m"], s["k"], 0.05, s["seed"], real=True)
        return srv.submit(s["n"], s["m"], s["k"], synthetic_j(s["n"]), weights=w, h=s["h"], seed=s["seed"],
                          chains=chains, samples_per_chain=m, burn_in=8, reglam0=5.0, tol=1e-12, max_steps=steps,
                          precision=s["prec"])

    alone = {}
    for s, args in ((big, (6, 256, 100)), (small, (6, 16, 20))):
        srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=4)
        submit(srv, s, *args)
        (r,) = srv.wait_all(1)
        srv.close()
        assert r["status"] == 0
        alone[s["seed"]] = r
    srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=4)
    id_big = submit(srv, big, 6, 256, 100)
    id_small = submit(srv, small, 6, 16, 20)
    order = [r["id"] for r in srv.wait_all(2)]
    srv.close()
    assert order == [id_small, id_big], order
    srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=4)
    ids = [submit(srv, big, 6, 256, 100), submit(srv, small, 6, 16, 20)]
    res = {r["id"]: r for r in srv.wait_all(2)}
    srv.close()
    for rid, s in zip(ids, (big, small)):
        a = alone[s["seed"]]
        assert res[rid]["energies"] == a["energies"] and res[rid]["steps"] == a["steps"]


@pytest.mark.gpu
def test_nonfinite_solve_restarts_then_fails_beside_a_healthy_one(pkg):
    """A solve whose weights hold a NaN goes non-finite at every step: the
    server restarts its run with a new seed 15 times (16 runs, as code/run.sh)
    and then fails it with NQES_ERR_NONFINITE, while a solve of another size
    class that runs at the same time (MIXED, the decision-warp sampler) is
    unaffected: its result equals running it alone."""
    bad = dict(n=20, m=40, k=3, h=0.8, prec=1, seed=71)
    good = dict(n=48, m=96, k=2, h=0.7, prec=1, seed=73)  # P = 9408: another lane

    def submit(srv, s, nan):
        a, b, w = helpers.random_weights(s["n"], s["m"], s["k"], 0.05, s["seed"], real=True)
        if nan:
            w[0, 1, 2] = np.nan
        return srv.submit(s["n"], s["m"], s["k"], synthetic_j(s["n"]), weights=(a, b, w), h=s["h"], seed=s["seed"],
                          chains=32, samples_per_chain=20, burn_in=8, reglam0=5.0, tol=1e-12, max_steps=4,
                          precision=s["prec"])

    srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=4)
    submit(srv, good, False)
    (alone,) = srv.wait_all(1)
    srv.close()
    assert alone["status"] == 0
    srv = pkg.Server(hbm_budget_bytes=1 << 36, max_active=4)
    id_bad = submit(srv, bad, True)
    id_good = submit(srv, good, False)
    res = {r["id"]: r for r in srv.wait_all(2)}
    err = srv.last_error()
    srv.close()
    rb, rg = res[id_bad], res[id_good]
    assert rb["status"] == pkg.ERR_NONFINITE and rb["restarts"] == 15, (rb, err)
    assert rg["status"] == 0 and rg["restarts"] == 0
    assert rg["energies"] == alone["energies"] and rg["steps"] == alone["steps"]
