"""Pins the CPU oracle against the golden fixtures (no GPU).

ref_golden.json comes from the reference's own pcg_random.h / minresqlp.h;
physics_golden.json from direct numpy evaluation of the definitions in
code/rbm.cc; ed_golden.json from exact diagonalisation."""
import json
import os

import numpy as np
import pytest

import helpers
from helpers import GOLDEN, Oracle, cfg_words, cplx_arr, dptr, synthetic_j, uptr


@pytest.fixture(scope="module")
def ref():
    with open(os.path.join(GOLDEN, "ref_golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="module")
def phys():
    with open(os.path.join(GOLDEN, "physics_golden.json")) as f:
        return json.load(f)


def test_pcg64_raw_uniform_bernoulli(ref, oracle_lib):
    for case in ref["rng"]:
        seed = int(case["seed"])
        n = len(case["raw"])
        raw = np.zeros(n, np.uint64)
        oracle_lib.orc_pcg64(seed, n, uptr(raw))
        assert [int(x) for x in raw] == [int(x) for x in case["raw"]]
        u = np.zeros(n)
        oracle_lib.orc_uniform(seed, n, dptr(u))
        assert np.array_equal(u, np.array(case["uniform"]))  # bit-exact
        b = np.zeros(n, np.uint8)
        import ctypes
        oracle_lib.orc_bernoulli(seed, n, b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
        assert np.array_equal(b, np.array(case["bernoulli"], np.uint8))


def test_pcg64_long_stream_checksums(ref, oracle_lib):
    for case in ref["rng"][:3]:
        seed = int(case["seed"])
        raw = np.zeros(1_000_000, np.uint64)
        oracle_lib.orc_pcg64(seed, raw.size, uptr(raw))
        s = int(np.sum(raw, dtype=np.uint64))  # wraps mod 2^64
        x = int(np.bitwise_xor.reduce(raw))
        assert s == int(case["sum1e6"]) and x == int(case["xor1e6"])
        u = np.zeros(1_000_000)
        oracle_lib.orc_uniform(seed, u.size, dptr(u))
        acc = 0.0
        for v in u:  # sequential sum, same order as the harness
            acc += float(v)
        assert acc == case["usum1e6"]


def test_reference_weight_init(ref):
    g = ref["init"]
    o = Oracle(g["N"], g["M"], g["K"], np.zeros((g["N"], g["N"])), 0.0)
    o.init_weights(g["seed"])
    a, b, w = o.get_weights()
    got = np.concatenate([np.concatenate([a[k], b[k], w[k].ravel()]) for k in range(g["K"])])
    want = cplx_arr(g["weights"])
    assert np.array_equal(got, want)


def test_minresqlp_matches_reference_solver(ref, oracle_lib):
    for case in ref["minresqlp"]:
        n = case["n"]
        A = np.array(case["A"])
        b = np.array(case["b"])
        x = np.zeros(2 * n)
        info = np.zeros(4)
        flag = oracle_lib.orc_minresqlp_dense(n, dptr(A), dptr(b), case["rtol"], int(case["maxit"]), dptr(x),
                                              dptr(info))
        assert flag == case["flag"]
        xr = cplx_arr(case["x"])
        xo = x.view(np.complex128)
        assert np.linalg.norm(xo - xr) <= 1e-9 * max(1.0, np.linalg.norm(xr))


def _case_oracle(case):
    o = Oracle(case["N"], case["M"], case["K"], np.array(case["J"]).reshape(case["N"], case["N"]), case["h"])
    K, N, M = case["K"], case["N"], case["M"]
    o.set_weights(cplx_arr(case["a"]).reshape(K, N), cplx_arr(case["b"]).reshape(K, M),
                  cplx_arr(case["w"]).reshape(K, N, M))
    return o


def test_oracle_physics_against_definitions(phys):
    for case in phys["cases"]:
        o = _case_oracle(case)
        for c in case["configs"]:
            words = cfg_words(c["cfg"], case["N"])
            phi, _ = o.state(words)
            want_phi = cplx_arr(c["phi"]).reshape(case["K"], case["K"])
            assert np.allclose(phi, want_phi, rtol=1e-12, atol=0)
            E, O = o.local(words)
            want_E = cplx_arr(c["E"]).reshape(case["K"], case["K"])
            assert np.max(np.abs(E - want_E)) <= 1e-11 * max(1.0, np.max(np.abs(want_E)))
            want_O = cplx_arr(c["O"])
            got_O = O[::c["O_stride"]]
            assert np.max(np.abs(got_O - want_O)) <= 1e-11 * max(1.0, np.max(np.abs(want_O)))


def test_oracle_sv_is_hermitian_positive():
    """After a sampling pass, the matrix-free S is Hermitian and S - diag part >= 0."""
    N, M, K = 4, 8, 2
    o = Oracle(N, M, K, synthetic_j(N), 0.595)
    o.set_weights(*helpers.random_weights(N, M, K, 0.1, 3))
    o.sr_step(11, 8, 20, 8, 0.0, 0.0, 1e-10, 5)
    rng = np.random.default_rng(0)
    P = o.P
    u = rng.normal(size=P) + 1j * rng.normal(size=P)
    v = rng.normal(size=P) + 1j * rng.normal(size=P)
    Su, Sv = o.apply_S(u), o.apply_S(v)
    assert abs(np.vdot(v, Su) - np.vdot(Sv, u)) <= 1e-10 * abs(np.vdot(v, Su))
    assert np.vdot(u, Su).real >= -1e-12


@pytest.mark.slow
def test_oracle_sr_reaches_exact_diagonalisation():
    """N=4, K=2: SR training reaches the ED energies (per site) within VMC noise."""
    with open(os.path.join(GOLDEN, "ed_golden.json")) as f:
        ed = json.load(f)
    case = [c for c in ed["cases"] if c["N"] == 4][0]
    N, M, K = 4, 8, 2
    o = Oracle(N, M, K, synthetic_j(N), case["h"])
    o.set_weights(*helpers.random_weights(N, M, K, 0.1, 7))
    lr, reglam = 0.1, 10.0
    hist = []
    for it in range(120):
        emat, info = o.sr_step(1000 + it * 16, 16, 100, 16, max(lr, 0.01), max(reglam, 0.01), 1e-9, 2000)
        lr *= 0.99
        reglam *= 0.9
        ev = np.sort(np.linalg.eigvals(emat / N).real)
        hist.append(ev)
    final = np.mean(hist[-10:], axis=0)
    assert np.all(np.abs(final - np.array(case["evals_per_site"])) < 0.02), (final, case["evals_per_site"])
