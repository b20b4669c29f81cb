"""The drop-in executable rbm-matfree-N{N}-M{M}-K{K}-opt.

CPU tests: the command-line surface of the reference (code/rbm.cc:900-961
through code/argparse.h) — help, missing/invalid arguments (exit 255),
-c 0 (exit 1), unknown options — and the MAT v5 reader/writer against scipy.
GPU test: a short run whose printed energies, dumped weights and correlation
file agree with the CPU oracle driven through the same schedule."""
import os
import subprocess

import numpy as np
import pytest

import __graft_entry__ as ge
import helpers

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BIN = os.path.join(ROOT, "nqes-trapped-ion_gb300", "bin")


JMAT = os.path.join(ROOT, "nqes-trapped-ion_gb300", "cli", "jmat")


def reference_j(n):
    """The couplings the reference compiles into its trapped-ion executables
    (code/Jmat/Ising2d_N{n}_alpha1.0.mat), as committed beside the CLI."""
    return np.fromfile(os.path.join(JMAT, f"Ising2d_N{n}_alpha1.0.f64"), dtype="<f8").reshape(n, n)


@pytest.fixture(scope="module")
def exe():
    ge._load_build_module().build_cli([(8, 16, 2)])
    return os.path.join(BIN, "rbm-matfree-N8-M16-K2-opt")


def run(cmd, **kw):
    return subprocess.run(cmd, capture_output=True, text=True, timeout=600, **kw)


def test_help_lists_the_reference_options(exe):
    r = run([exe, "-?"])
    assert r.returncode == 0
    assert r.stdout.startswith("This program computes the lowest 2 energy eigenstates")
    for key in ["--model", "-n,--niters", "-m,--mc-steps-percpu", "-c,--ncpus", "--burn-in-steps", "--tol",
                "--reglam-init", "--reglam-cutoff", "--minres-rtol", "--correlation-data", "--dump-rbm",
                "--throw-fperror", "--load-rbm"]:
        assert key in r.stdout, key


def test_missing_and_invalid_arguments(exe):
    r = run([exe, "--model", "trappedion", "-h", "1", "-n", "2", "-m", "3"])
    assert r.returncode == 255
    assert r.stderr.strip() == "Argument missing: -c,--ncpus (Specify the number of CPU cores to use.)"
    r = run([exe, "--model", "nope", "-h", "1", "-n", "2", "-m", "3", "-c", "1", "--correlation-data", "x.mat"])
    assert r.returncode == 255
    assert "enum is only accepting [ising, periodicising, hs, xxz, longrange, trappedion]" in r.stderr
    r = run([exe, "--model", "TRAPPEDION", "-h", "abc", "-n", "2", "-m", "3", "-c", "1", "--correlation-data", "x"])
    assert r.returncode == 255 and r.stderr.startswith('Invalid argument, could not convert "abc" for -h')


def test_zero_chains_and_unknown_option(exe):
    r = run([exe, "--model", "trappedion", "-h", "1", "-n", "2", "-m", "3", "-c", "0", "--correlation-data", "x",
             "--bogus", "1"])
    assert r.returncode == 1
    assert "unrecognised commandline argument: bogus" in r.stderr
    assert "Number of CPU cores cannot be zero." in r.stderr


def test_compiled_in_couplings_are_the_reference_jmat(exe, tmp_path):
    """--model trappedion uses the reference's compiled-in J (code/build.sh:34-41,
    code/rbm.cc:1011-1031) element for element; --jmat synthetic the power-law
    chain of the benchmark inputs. --dump-jmat writes the J that nqes_create
    would receive and exits before touching a device."""
    sio = pytest.importorskip("scipy.io")
    base = [exe, "--model", "trappedion", "-h", "0.595", "-n", "1", "-m", "1", "-c", "1", "--correlation-data", "x"]
    f = str(tmp_path / "j.mat")
    r = run(base + ["--dump-jmat", f])
    assert r.returncode == 0, r.stderr
    J = sio.loadmat(f)["J"]
    assert np.array_equal(J, reference_j(8))
    ref = os.environ.get("NQES_REFERENCE_DIR")
    if ref and os.path.isdir(ref):  # the committed values against the reference's own file
        want = sio.loadmat(os.path.join(ref, "code", "Jmat", "Ising2d_N8_alpha1.0.mat"))["J"]
        assert np.array_equal(J, want)
    r = run(base + ["--jmat", "synthetic", "--dump-jmat", f])
    assert r.returncode == 0, r.stderr
    assert np.array_equal(sio.loadmat(f)["J"], helpers.synthetic_j(8))


@pytest.fixture(scope="module")
def mat_driver(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("drv") / "mat_driver")
    cli = os.path.join(ROOT, "nqes-trapped-ion_gb300", "cli")
    subprocess.run(["g++", "-std=c++20", "-O1", "-I", cli, os.path.join(ROOT, "tests", "mat_driver.cc"),
                    os.path.join(cli, "matv5.cc"), "-o", out], check=True)
    return out


def test_mat_reader_reads_scipy_files(mat_driver, tmp_path):
    sio = pytest.importorskip("scipy.io")
    rng = np.random.default_rng(0)
    a = rng.normal(size=(2, 5)) + 1j * rng.normal(size=(2, 5))
    w = rng.normal(size=(2, 5, 3)) + 1j * rng.normal(size=(2, 5, 3))
    J = rng.normal(size=(4, 4))
    f = str(tmp_path / "w.mat")
    sio.savemat(f, {"a": a, "w": w, "J": J, "N": 4})
    out = run([mat_driver, "read", f]).stdout.strip().split("\n")
    got = {ln.split()[0]: ln.split()[1:] for ln in out}
    for name, arr in [("a", a), ("w", w), ("J", J)]:
        fields = got[name]
        cpx, rank = int(fields[0]), int(fields[1])
        dims = tuple(int(d) for d in fields[2:2 + rank])
        vals = np.array([float(v) for v in fields[2 + rank:]])
        assert dims == arr.shape and cpx == int(np.iscomplexobj(arr))
        flat = arr.ravel(order="F")
        want = np.stack([flat.real, flat.imag], -1).ravel() if cpx else flat
        assert np.array_equal(vals, want)
    assert [float(v) for v in got["N"][4:]] == [4.0]


def test_mat_writer_is_read_by_scipy(mat_driver, tmp_path):
    sio = pytest.importorskip("scipy.io")
    f = str(tmp_path / "o.mat")
    assert run([mat_driver, "write", f]).returncode == 0
    d = sio.loadmat(f)
    want_a = (np.arange(6) + 0.25 - 1j * (np.arange(6) + 0.5)).reshape(2, 3, order="F")
    assert np.array_equal(d["a"], want_a)
    assert np.array_equal(d["xx"], (np.arange(8) * 1.5).reshape(2, 2, 2, order="F"))


@pytest.mark.gpu
def test_executable_matches_oracle_schedule(exe, tmp_path):
    sio = pytest.importorskip("scipy.io")
    N, M, K, h = 8, 16, 2, 0.595
    seed, chains, m, burn, niters = 31, 8, 25, 8, 4
    w0 = helpers.random_weights(N, M, K, 0.05, 2, real=False)
    wfile = str(tmp_path / "w0.mat")
    sio.savemat(wfile, {"a": w0[0], "b": w0[1], "w": w0[2]})
    corr = str(tmp_path / "corr.mat")
    prefix = str(tmp_path / "out")
    args = [exe, "--model", "trappedion", "-h", str(h), "-n", str(niters), "-m", str(m), "-c", str(chains),
            "--burn-in-steps", str(burn), "--seed", str(seed), "--load-rbm", wfile, "--reglam-init", "5",
            "--minres-rtol", "1e-9", "--tol", "1e-12", "--correlation-data", corr, "--dump-rbm", prefix]
    r = run(args)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().split("\n")
    assert lines[0] == f"Random seed is {seed}"
    got = np.array([[float(v) for v in ln.split()] for ln in lines[1:1 + niters]])
    # oracle through the same schedule (code/rbm.cc:1178-1196)
    orc = helpers.Oracle(N, M, K, reference_j(N), h)
    orc.set_weights(*w0)
    lr, reglam = 0.1, 5.0
    want = []
    for it in range(niters):
        e, _ = orc.sr_step(seed + it * chains, chains, m, burn, max(lr, 0.01), max(reglam, 0.001), 1e-9, 2 ** 63)
        e = e / N
        lr *= 0.99
        reglam *= 0.9
        want.append(np.sort(np.linalg.eigvals(e).real))
    want = np.array(want)
    assert np.allclose(got, want, rtol=0, atol=2e-5), (got, want)  # printed with 6 significant digits
    d = sio.loadmat(prefix + f"N{N}M{M}K{K}.mat")
    ao, bo, wo = orc.get_weights()
    assert np.max(np.abs(d["w"] - wo)) <= 1e-5 * np.max(np.abs(wo))
    # correlations with the oracle's own eigenvectors of the last e_mat, sorted by eigenvalue
    ev, V = np.linalg.eig(e)
    order = np.argsort(ev.real)
    x, z, xx, zz = orc.correlations(seed + niters * chains, chains, m, burn, V)
    c = sio.loadmat(corr)
    assert np.allclose(c["x"], x[:, order], atol=1e-6)
    assert np.allclose(c["z"], z[:, order], atol=1e-6)
    assert np.allclose(c["xx"], xx[:, order].reshape(N, N, K), atol=1e-6)
    assert np.allclose(c["zz"], zz[:, order].reshape(N, N, K), atol=1e-6)


@pytest.mark.gpu
@pytest.mark.parametrize("model", ["xxz", "hs"])
def test_executable_heisenberg_models(exe, tmp_path, model):
    """--model xxz / hs (code/rbm.cc:1064-1119, 1314-1325): the printed
    energies follow the oracle through the same schedule."""
    sio = pytest.importorskip("scipy.io")
    from test_oracle_heisenberg import hs_j, xxz_j
    N, M, K = 8, 16, 2
    seed, chains, m, burn, niters = 17, 8, 25, 8, 3
    w0 = helpers.random_weights(N, M, K, 0.05, 4, real=False)
    wfile = str(tmp_path / "w0.mat")
    sio.savemat(wfile, {"a": w0[0], "b": w0[1], "w": w0[2]})
    args = [exe, "--model", model, "-h", "0", "-n", str(niters), "-m", str(m), "-c", str(chains), "--burn-in-steps", str(burn),
            "--seed", str(seed), "--load-rbm", wfile, "--reglam-init", "5", "--minres-rtol", "1e-9", "--tol", "1e-12",
            "--correlation-data", str(tmp_path / "corr.mat"), "--dump-rbm", str(tmp_path / "out")]
    r = run(args)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().split("\n")
    got = np.array([[float(v) for v in ln.split()] for ln in lines[1:1 + niters]])
    J, delta = (hs_j(N), 1.0) if model == "hs" else (xxz_j(N), -1.0)
    orc = helpers.Oracle(N, M, K, J, 0.0)
    orc.set_hamiltonian(1, delta)
    orc.set_weights(*w0)
    lr, reglam = 0.1, 5.0
    want = []
    for it in range(niters):
        e, _ = orc.sr_step(seed + it * chains, chains, m, burn, max(lr, 0.01), max(reglam, 0.001), 1e-9, 2 ** 63)
        lr *= 0.99
        reglam *= 0.9
        want.append(np.sort(np.linalg.eigvals(e / N).real))
    assert np.allclose(got, np.array(want), rtol=0, atol=2e-5), (got, want)


@pytest.mark.gpu
def test_executable_dumps(exe, tmp_path):
    """--dump-states / --dump-ham / --dump-deriv (code/rbm.cc:473-524,
    1150-1172): Phi, E and O at all 2^(K N) configurations in the reference's
    MAT layout (variable s, [2^(KN), rows, cols], column-major), against the
    oracle at sampled configurations (the E of configurations with equal rows,
    where the reference takes a pseudo-inverse, is checked in test_gpu_edges)."""
    sio = pytest.importorskip("scipy.io")
    N, M, K, h, seed = 8, 16, 2, 0.595, 5
    w0 = helpers.random_weights(N, M, K, 0.05, 6, real=False)
    wfile = str(tmp_path / "w0.mat")
    sio.savemat(wfile, {"a": w0[0], "b": w0[1], "w": w0[2]})
    pre = {k: str(tmp_path / k) for k in ("st", "ham", "der")}
    args = [exe, "--model", "trappedion", "-h", str(h), "-n", "1", "-m", "4", "-c", "2", "--burn-in-steps", "2",
            "--seed", str(seed), "--load-rbm", wfile, "--correlation-data", str(tmp_path / "corr.mat"),
            "--dump-rbm", str(tmp_path / "out"), "--dump-states", pre["st"], "--dump-ham", pre["ham"],
            "--dump-deriv", pre["der"]]
    r = run(args)
    assert r.returncode == 0, r.stderr
    suffix = f"N{N}M{M}K{K}.mat"
    st = sio.loadmat(pre["st"] + suffix)["s"]
    ham = sio.loadmat(pre["ham"] + suffix)["s"]
    der = sio.loadmat(pre["der"] + suffix)["s"]
    P = K * (N + M + N * M)
    assert st.shape == (2 ** (K * N), K, K) and ham.shape == (2 ** (K * N), K, K) and der.shape == (2 ** (K * N), P)
    orc = helpers.Oracle(N, M, K, reference_j(N), h)
    orc.set_weights(*w0)
    rng = np.random.default_rng(1)
    for idx in list(rng.integers(0, 2 ** (K * N), size=12)) + [0x1234, 2 ** (K * N) - 2]:
        idx = int(idx)
        rows = [(idx >> (k * N)) & ((1 << N) - 1) for k in range(K)]
        if rows[0] == rows[1]:
            continue
        words = np.array([[r] for r in rows], dtype=np.uint64)
        phi, _ = orc.state(words)
        E, O = orc.local(words)
        assert np.max(np.abs(st[idx] - phi)) <= 1e-12 * np.max(np.abs(phi))
        assert np.max(np.abs(ham[idx] - E)) <= 1e-10 * np.max(np.abs(E))
        assert np.max(np.abs(der[idx] - O)) <= 1e-10 * np.max(np.abs(O))


@pytest.mark.gpu
def test_nonfinite_weights_exit_127_with_throw_fperror(exe, tmp_path):
    """A NaN weight loaded with --load-rbm makes the first SR step non-finite:
    with --throw-fperror the executable exits with status 127, the code
    run.sh retries on (code/rbm.cc:1248-1271); without it the run carries on
    and exits 0, as the reference does with floating-point traps off."""
    sio = pytest.importorskip("scipy.io")
    N, M, K = 8, 16, 2
    a, b, w = helpers.random_weights(N, M, K, 0.05, 8, real=False)
    w[1, 3, 5] = np.nan
    wfile = str(tmp_path / "nan.mat")
    sio.savemat(wfile, {"a": a, "b": b, "w": w})
    base = [exe, "--model", "trappedion", "-h", "0.595", "-n", "2", "-m", "4", "-c", "2", "--burn-in-steps", "2",
            "--seed", "3", "--load-rbm", wfile, "--correlation-data", str(tmp_path / "c.mat")]
    r = run(base + ["--throw-fperror"])
    assert r.returncode == 127, (r.returncode, r.stderr)
    assert "Floating point error occured. Exiting." in r.stderr
    r = run(base)
    assert r.returncode == 0, (r.returncode, r.stderr)
