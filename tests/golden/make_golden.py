"""Generates the committed golden fixtures under tests/golden/.

Run from the repository root:  python tests/golden/make_golden.py [--reference DIR] [--only ref|physics|ed]
(DIR defaults to the environment variable NQES_REFERENCE_DIR.)

1. ref_golden.json — outputs of the reference's own header-only code
   (code/pcg_random.h, code/minresqlp.h, compiled where they lie by
   `make -C oracle ref`): pcg64 raw streams, libstdc++ uniform/Bernoulli draws on
   them (code/rbm.cc:103,535), long-stream checksums, the reference weight
   initialisation order (code/rbm.cc:241-270), and MINRES-QLP solutions of
   seeded Hermitian systems. Needs the reference tree; skipped without it.
2. physics_golden.json — Phi, E = Phi^-1 H Phi and O = d log det Phi / dW at
   fixed configurations and complex weights, evaluated in numpy directly from
   the definitions stated in code/rbm.cc (amplitude 134-171, Hamiltonian
   1011-1062 with H = sum_{i!=j} J_ij sz_i sz_j - h sum_i sx_i, derivatives
   192-239), independently of the C++ oracle. O is checked here against a
   holomorphic finite difference of log det Phi before it is written.
3. ed_golden.json — the K lowest eigenvalues per site of H (exact
   diagonalisation, scipy) for the synthetic power-law chains used by tests
   (N up to 20) and for the reference's own 2D ion-crystal couplings
   (code/Jmat/Ising2d_N{8,16}_alpha1.0.mat).
"""
import argparse
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def synthetic_j(n, alpha=1.2):
    """J_ij = |i-j|^-alpha (i != j), 0 on the diagonal; max |J| = 1."""
    i = np.arange(n)
    d = np.abs(i[:, None] - i[None, :]).astype(float)
    with np.errstate(divide="ignore"):
        J = np.where(d > 0, d ** (-alpha), 0.0)
    return J / np.max(np.abs(J)) if n > 1 else J


def sigma(bits, n):
    """sigma_i = +1 for bit 0, -1 for bit 1 (code/rbm.cc:138-141)."""
    return np.array([-1.0 if (bits >> i) & 1 else 1.0 for i in range(n)])


def psi(a, b, w, s):
    """Unnormalised RBM amplitude exp(a.s) prod_j cosh(b_j + sum_i s_i w_ij)."""
    return np.exp(a @ s) * np.prod(np.cosh(b + s @ w))


def grand_phi(a, b, w, cfg, n):
    K = a.shape[0]
    P = np.empty((K, K), complex)
    for k in range(K):
        s = sigma(cfg[k], n)
        for kk in range(K):
            P[k, kk] = psi(a[kk], b[kk], w[kk], s)
    return P


def h_phi(a, b, w, cfg, n, J, h):
    """(H Phi)[k, kk] = sum_s' <s_k|H|s'> psi_kk(s')."""
    K = a.shape[0]
    out = np.empty((K, K), complex)
    for k in range(K):
        s = sigma(cfg[k], n)
        diag = sum(J[i, j] * s[i] * s[j] for i in range(n) for j in range(n) if i != j)
        for kk in range(K):
            v = diag * psi(a[kk], b[kk], w[kk], s)
            for i in range(n):
                v -= h * psi(a[kk], b[kk], w[kk], sigma(cfg[k] ^ (1 << i), n))
            out[k, kk] = v
    return out


def log_derivs(a, b, w, cfg, n):
    """O_{k,p} = d log det Phi / d W_{k,p}, layout [k][a_i | b_j | w_{i*M+j}]."""
    K, M = b.shape
    P = grand_phi(a, b, w, cfg, n)
    Pinv = np.linalg.inv(P)
    L = n + M + n * M
    O = np.empty(K * L, complex)
    for k in range(K):
        # d Phi[kk, k] / d W_{k,p} = Phi[kk, k] * d_p(s_kk); chain rule through det.
        ds = []
        for kk in range(K):
            s = sigma(cfg[kk], n)
            t = np.tanh(b[k] + s @ w[k])
            ds.append(np.concatenate([s, t, np.outer(s, t).ravel()]))
        ds = np.array(ds)  # K x L
        coef = np.array([Pinv[k, kk] * P[kk, k] for kk in range(K)])
        O[k * L:(k + 1) * L] = coef @ ds
    return O


def fd_check(a, b, w, cfg, n, O):
    """Holomorphic central difference of log det Phi along a random direction."""
    rng = np.random.default_rng(5)
    K, M = b.shape
    L = n + M + n * M
    da = rng.normal(size=a.shape) + 1j * rng.normal(size=a.shape)
    db = rng.normal(size=b.shape) + 1j * rng.normal(size=b.shape)
    dw = rng.normal(size=w.shape) + 1j * rng.normal(size=w.shape)
    eps = 1e-6
    f = lambda t: np.log(np.linalg.det(grand_phi(a + t * da, b + t * db, w + t * dw, cfg, n)))
    num = (f(eps) - f(-eps)) / (2 * eps)
    dirv = np.concatenate([np.concatenate([da[k], db[k], dw[k].ravel()]) for k in range(K)])
    ana = O @ dirv
    assert abs(num - ana) <= 1e-6 * max(1.0, abs(ana)), (num, ana)


def make_physics():
    cases = []
    specs = [  # (N, M, K, h, weight scale, seed, n_configs)
        (4, 8, 2, 0.595, 0.3, 1, 6),
        (5, 5, 3, 1.0, 0.25, 2, 5),
        (6, 12, 1, 0.7, 0.2, 3, 4),
        (7, 14, 4, 0.4, 0.15, 4, 4),
        (66, 66, 2, 0.595, 0.05, 6, 1),
    ]
    for (n, M, K, h, sc, seed, ncfg) in specs:
        rng = np.random.default_rng(seed)
        a = sc * (rng.normal(size=(K, n)) + 1j * rng.normal(size=(K, n)))
        b = sc * (rng.normal(size=(K, M)) + 1j * rng.normal(size=(K, M)))
        w = sc * (rng.normal(size=(K, n, M)) + 1j * rng.normal(size=(K, n, M))) / np.sqrt(n)
        J = synthetic_j(n)
        cfgs = []
        while len(cfgs) < ncfg:
            cfg = [sum(int(bit) << i for i, bit in enumerate(rng.integers(0, 2, size=n))) for _ in range(K)]
            if len(set(cfg)) < K:
                continue
            cfgs.append(cfg)
        out = []
        for cfg in cfgs:
            P = grand_phi(a, b, w, cfg, n)
            E = np.linalg.solve(P, h_phi(a, b, w, cfg, n, J, h))
            O = log_derivs(a, b, w, cfg, n)
            if n <= 8:
                fd_check(a, b, w, cfg, n, O)
            # Wide cases keep every 13th log-derivative to stay small.
            stride = 1 if n <= 8 else 13
            Os = O[::stride]
            out.append({
                "cfg": [str(c) for c in cfg],
                "phi": np.stack([P.real, P.imag], -1).ravel().tolist(),
                "E": np.stack([E.real, E.imag], -1).ravel().tolist(),
                "O_stride": stride,
                "O": np.stack([Os.real, Os.imag], -1).ravel().tolist(),
            })
        cplx = lambda z: np.stack([z.real, z.imag], -1).ravel().tolist()
        cases.append({"N": n, "M": M, "K": K, "h": h, "J": J.ravel().tolist(),
                      "a": cplx(a), "b": cplx(b), "w": cplx(w), "configs": out})
    return {"cases": cases}


def reference_j(n):
    """The reference's compiled-in couplings code/Jmat/Ising2d_N{n}_alpha1.0.mat,
    as extracted to nqes-trapped-ion_gb300/cli/jmat/ (raw float64, row-major)."""
    path = os.path.join(ROOT, "nqes-trapped-ion_gb300", "cli", "jmat", f"Ising2d_N{n}_alpha1.0.f64")
    return np.fromfile(path, dtype="<f8").reshape(n, n)


# (N, h, K, couplings): "alpha1.2" is the power-law chain above, "ion2d" the
# reference's 2D ion-crystal J of the same N.
ED_CASES = [(4, 0.595, 2, "alpha1.2"), (6, 0.595, 2, "alpha1.2"), (8, 0.595, 2, "alpha1.2"), (8, 1.0, 3, "alpha1.2"),
            (10, 0.595, 2, "alpha1.2"), (12, 0.595, 2, "alpha1.2"), (16, 0.595, 2, "alpha1.2"),
            (20, 0.595, 2, "alpha1.2"), (8, 0.595, 2, "ion2d"), (16, 0.595, 2, "ion2d")]


def make_ed():
    """K lowest eigenvalues per site of H = sum_{i!=j} J_ij sz_i sz_j - h sum_i sx_i
    (the reference's ising_like_hamiltonian with J(s) = 2 sum_{i>j} J_ij s_i s_j,
    code/rbm.cc:1011-1062): dense eigvalsh up to 1024 states, else Lanczos
    (scipy eigsh) on a matrix-free H."""
    import scipy.sparse.linalg as sla
    out = []
    for (n, h, K, kind) in ED_CASES:
        J = synthetic_j(n) if kind == "alpha1.2" else reference_j(n)
        dim = 1 << n
        idx = np.arange(dim)
        diag = np.zeros(dim)
        for i in range(n):
            si = 1.0 - 2.0 * ((idx >> i) & 1)
            for j in range(i):
                sj = 1.0 - 2.0 * ((idx >> j) & 1)
                diag += 2.0 * J[i, j] * si * sj

        def matvec(x):
            x = np.asarray(x).ravel()
            y = diag * x
            for i in range(n):
                y -= h * x[idx ^ (1 << i)]
            return y

        if dim <= 1024:
            H = np.stack([matvec(np.eye(dim)[c]) for c in range(dim)], 1)
            ev = np.sort(np.linalg.eigvalsh(H))[:K]
        else:
            op = sla.LinearOperator((dim, dim), matvec=matvec, dtype=np.float64)
            ev = np.sort(sla.eigsh(op, k=K, which="SA", tol=1e-12)[0])
        case = {"N": n, "h": h, "K": K, "couplings": kind, "evals_per_site": (ev / n).tolist()}
        if kind == "alpha1.2":
            case["alpha"] = 1.2
        out.append(case)
    return {"cases": out}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("NQES_REFERENCE_DIR"),
                    help="the reference tree (default: $NQES_REFERENCE_DIR)")
    ap.add_argument("--only", choices=["ref", "physics", "ed"], help="regenerate one file only")
    args = ap.parse_args()
    if args.only in (None, "ref") and args.reference and os.path.isdir(args.reference):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={args.reference}"], check=True)
        raw = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_harness")], check=True,
                             capture_output=True, text=True).stdout
        data = json.loads(raw)
        with open(os.path.join(HERE, "ref_golden.json"), "w") as f:
            json.dump(data, f, separators=(",", ":"))
    elif args.only in (None, "ref"):
        print("reference tree absent: ref_golden.json left as committed", file=sys.stderr)
    if args.only in (None, "physics"):
        with open(os.path.join(HERE, "physics_golden.json"), "w") as f:
            json.dump(make_physics(), f, separators=(",", ":"))
    if args.only in (None, "ed"):
        with open(os.path.join(HERE, "ed_golden.json"), "w") as f:
            json.dump(make_ed(), f, indent=1)


if __name__ == "__main__":
    main()
