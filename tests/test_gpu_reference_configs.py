"""GPU against the oracle at the benchmark's own configurations, and against
the reference's published data.

* One FP64 SR step at exactly N8 M16 K2 and N32 M64 K2 (h = 0.595,
  J_ij = |i-j|^-1.2, seeded real N(0, 0.01^2) weights, 128 chains x 200
  samples, burn-in 64, lambda 40, lr 0.1, MINRES-QLP rtol 1e-9): every sampled
  configuration bit-identical, the accept count equal, e_mat, o and S·v
  within 1e-12 relative (norm-wise: the largest difference over the largest
  entry), the quantities that pass through Phi^-1 of the benchmark's nearly
  rank-one Phi within 1e-11 (see the test), the MINRES-QLP flag equal and
  its iteration count equal or one apart.
* One complex SR step on the reference's trained weights
  data/rbm-weights/ionh0.595train1.2N50M150K2.mat with its compiled-in
  couplings code/Jmat/Ising2d_N50_alpha1.0.mat (committed as fixtures), same
  checks.
* The drop-in executable rbm-matfree-N50-M150-K2-opt run on the reference's
  trained weights (--load-rbm) against the per-site energies that the
  reference printed over the last 20 SR steps of the run that produced them
  (data/energy/ion_N50_M150_K2_h0.595_c128_m200-{1,2}): within 1 % relative.
  The measured gap is 0.3-0.5 %, our energies above the logged ones, with the
  same sign and size for the reference's Ising N128 weights (no J file
  involved) and when a run's first printed line is recomputed from the
  weights it loaded and its printed seed. The GPU and the CPU restatement of
  code/rbm.cc agree with each other to 1e-12 on these weights and to
  Monte Carlo noise on these energies, so the gap lies between the source
  restated here and the binary that wrote the logs, which cannot be built
  here (no Eigen3 or libmatio). This test pins the drop-in path (the loaded
  MAT layout, the compiled-in couplings, h, the estimator) at that level.
"""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import __graft_entry__ as ge
import helpers
from helpers import GOLDEN, Oracle, synthetic_j

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
JMAT = os.path.join(ROOT, "nqes-trapped-ion_gb300", "cli", "jmat")
BIN = os.path.join(ROOT, "nqes-trapped-ion_gb300", "bin")
SEED = 20240601


@pytest.fixture(scope="module")
def pkg():
    ge._load_build_module().build_library()
    return ge.load_package()


def rel_err(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def reference_j(n):
    return np.fromfile(os.path.join(JMAT, f"Ising2d_N{n}_alpha1.0.f64"), dtype="<f8").reshape(n, n)


def trained_weights(index):
    z = np.load(os.path.join(GOLDEN, "ref_trained_N50M150K2.npz"))
    return z[f"a{index}"], z[f"b{index}"], z[f"w{index}"]


def step_and_compare(pkg, N, M, K, J, h, weights, chains, m, burn, lr, reglam, rtol, seed, tol, o_rows, tols=None,
                     iters_slack=0.0):
    ctx = pkg.Context(N, M, K, J, h)
    ctx.set_weights(*weights)
    orc = Oracle(N, M, K, J, h)
    orc.set_weights(*weights)
    args = (seed, chains, m, burn, lr, reglam, rtol, 100000)
    e_g, info = ctx.sr_step(*args)
    e_o, oinfo = orc.sr_step(*args, store_o=True)
    ns = chains * m
    sg, elg, Eg = ctx.get_samples()
    so, elo, Eo = orc.samples(ns)
    assert np.array_equal(sg, so), "sampled configurations differ"
    assert info["accepted"] == int(oinfo["accepted"])
    errs = {"E": rel_err(Eg, Eo), "eloc": rel_err(elg, elo), "e_mat": rel_err(e_g, e_o)}
    og, sk_g, fg = ctx.get_moments()
    oo, sk_o, fo = orc.moments()
    errs.update(o=rel_err(og, oo), skk=rel_err(sk_g, sk_o), f=rel_err(fg, fo))
    rows = np.unique(np.linspace(0, ns - 1, o_rows).astype(int))
    errs["O"] = max(rel_err(ctx.get_O(int(s), 1)[0], orc.sample_deriv(int(s))) for s in rows)
    rng = np.random.default_rng(5)
    real = info["arith"] == pkg.ARITH_REAL
    v = rng.normal(size=ctx.P) + (0 if real else 1j) * rng.normal(size=ctx.P)
    errs["Sv"] = rel_err(ctx.apply_S(v), orc.apply_S(v))
    print({k: f"{x:.2e}" for k, x in errs.items()}, "iters", info["minres_iters"], int(oinfo["iters"]))
    for k, x in errs.items():
        assert x < (tols or {}).get(k, tol), (k, x)
    assert info["minres_flag"] == int(oinfo["flag"])
    it_g, it_o = int(info["minres_iters"]), int(oinfo["iters"])
    assert abs(it_g - it_o) <= iters_slack * it_o, (it_g, it_o)
    # the solution meets the reference's relative-residual bound with the oracle's S
    x = ctx.get_solution()
    r = np.linalg.norm(orc.apply_S(x) - fo)
    assert r <= 10 * rtol * (info["anorm"] * np.linalg.norm(x) + np.linalg.norm(fo)), r
    ctx.close()
    return info


@pytest.mark.parametrize("N,M", [(8, 16), (32, 64)], ids=["N8M16K2", "N32M64K2"])
def test_benchmark_configuration_step(pkg, N, M):
    K = 2
    w = pkg.synthetic_weights(N, M, K, 0.01, SEED)
    # With N(0, 0.01^2) weights the K RBMs are within about 1 % of each other,
    # so Phi is nearly rank one and what Phi^-1 enters (the per-sample E and
    # its trace, the log-derivative rows, and f = <E O> - <E><O>, a centred
    # difference of them) carries rounding amplified by cond(Phi) ~ 1e2: 1e-11
    # there (measured 1-5e-12, E up to 1e-11: 2e-11). The averages e_mat and
    # o, the regularised diagonal and S·v meet 1e-12 (measured <= 1e-12), and
    # the trained weights below, whose Phi is well conditioned, meet 1e-12 in
    # every quantity.
    # MINRES-QLP: the same exit flag; the iteration count equal or, where the
    # relative residual crosses rtol within rounding at the last iteration,
    # one apart (measured: equal at N32 M64 K2, equal or one apart at N8 M16 K2).
    info = step_and_compare(pkg, N, M, K, synthetic_j(N), 0.595, w, 128, 200, 64, 0.1, 40.0, 1e-9, SEED,
                            1e-12, 64, tols={"E": 2e-11, "eloc": 1e-11, "O": 1e-11, "f": 1e-11, "skk": 2e-12},
                            iters_slack=1.5 / 60)
    assert info["arith"] == pkg.ARITH_REAL


def test_reference_trained_weights_complex_step(pkg):
    N, M, K = 50, 150, 2
    # 128 samples for 15400 parameters: S is the regularised diagonal plus a
    # rank-128 term, and the Krylov iteration count (several hundred) moves
    # with the last bits of S·v; flag, energies and moments do not.
    info = step_and_compare(pkg, N, M, K, reference_j(N), 0.595, trained_weights(0), 8, 16, 16, 0.01, 1.0, 1e-9,
                            929051268, 1e-12, 16, iters_slack=0.05)
    assert info["arith"] == pkg.ARITH_COMPLEX


@pytest.mark.parametrize("run", [0, 1])
def test_executable_reproduces_reference_energies(pkg, tmp_path, run):
    sio = pytest.importorskip("scipy.io")
    with open(os.path.join(GOLDEN, "ref_energy_tails.json")) as f:
        fx = json.load(f)
    r = fx["runs"][run]
    exe = ge._load_build_module().build_cli([(50, 150, 2)])[0]
    a, b, w = trained_weights(r["npz_index"])
    wfile = str(tmp_path / "w.mat")
    sio.savemat(wfile, {"a": a, "b": b, "w": w})
    steps = 4
    # the reference's flags for this run, with the learning rate at zero so
    # that every step samples the loaded weights (independent seeds per step)
    cmd = [exe, "-c", "128", "--model", "trappedion", "-h", "0.595", "-n", str(steps), "-m", "200", "--tol", "0",
           "--reglam-init", "40", "--reglam-cutoff", "1", "--minres-rtol", "1e-9", "--lrate-init", "0",
           "--lrate-cutoff", "0", "--seed", str(4242 + run), "--load-rbm", wfile,
           "--correlation-data", str(tmp_path / "c.mat")]
    p = subprocess.run(cmd, capture_output=True, text=True, timeout=1200)
    assert p.returncode == 0, p.stderr
    lines = [ln for ln in p.stdout.split("\n") if re.match(r"^\s*-?\d", ln)]
    ours = np.array([[float(x) for x in ln.split()] for ln in lines])
    assert ours.shape == (steps, 2), p.stdout
    ref = np.array(r["energies_per_site"])
    rel = (ours.mean(0) - ref.mean(0)) / np.abs(ref.mean(0))
    print("ours", ours.mean(0), "reference", ref.mean(0), "relative gap", rel)
    assert np.all(np.abs(rel) < 0.01), (ours.mean(0), ref.mean(0), rel)
