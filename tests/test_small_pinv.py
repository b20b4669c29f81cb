"""small_pinv (nqes_math.cuh), the Moore-Penrose pseudo-inverse that the
evaluation path takes at rank-deficient Phi (the reference's
completeOrthogonalDecomposition().pseudoInverse(), code/rbm.cc:547, 608),
compiled for the host and checked against numpy.linalg.pinv on matrices of
every rank for K = 1..4, complex and real, including exactly repeated rows."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "nqes-trapped-ion_gb300", "csrc")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path_factory.mktemp("pinv") / "pinv_harness")
    subprocess.run(["nvcc", "-std=c++17", "-O2", "-I", CSRC, "-o", exe,
                    os.path.join(ROOT, "tests", "pinv_harness.cu")], check=True)
    return exe


def matrices(K, rng):
    out = []
    for r in range(K + 1):
        for real in (False, True):
            for _ in range(3):
                U = rng.normal(size=(K, r)) + (0 if real else 1j) * rng.normal(size=(K, r))
                V = rng.normal(size=(K, r)) + (0 if real else 1j) * rng.normal(size=(K, r))
                out.append((U @ V.conj().T * 10.0 ** rng.uniform(-3, 3), r))
    if K > 1:  # exactly repeated rows of a full-rank matrix
        A = rng.normal(size=(K, K)) + 1j * rng.normal(size=(K, K))
        A[1] = A[0]
        out.append((A, K - 1))
    return out


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_small_pinv_matches_numpy(harness, K):
    rng = np.random.default_rng(K)
    cases = matrices(K, rng)
    text = f"{len(cases)} {K}\n" + "\n".join(" ".join("%.17g %.17g" % (z.real, z.imag) for z in A.ravel()) for A, _ in cases)
    res = subprocess.run([harness], input=text, capture_output=True, text=True, check=True)
    lines = res.stdout.strip().split("\n")
    assert len(lines) == len(cases)
    for (A, r), ln in zip(cases, lines):
        v = ln.split()
        rank = int(v[0])
        P = (np.array([float(x) for x in v[1::2]]) + 1j * np.array([float(x) for x in v[2::2]])).reshape(K, K)
        assert rank == r, (rank, r)
        want = np.linalg.pinv(A)
        scale = max(np.max(np.abs(want)), 1e-300)
        assert np.max(np.abs(P - want)) <= 1e-9 * scale, (r, np.max(np.abs(P - want)) / scale)
