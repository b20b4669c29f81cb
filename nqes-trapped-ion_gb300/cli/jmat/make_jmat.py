"""Extracts the reference's compiled-in trapped-ion couplings.

    python nqes-trapped-ion_gb300/cli/jmat/make_jmat.py [--reference DIR]

The reference compiles J into each executable: code/build.sh:34-41 runs
code/load_jmat.py N, which prints Jmat[N][N] from
code/Jmat/Ising2d_N{N}_alpha1.0.mat (variable J, the 2D ion-crystal couplings
with alpha = 1.0), and code/rbm.cc:1011-1031 sums it. This script reads the
same MAT files (scipy.io.loadmat) and writes each J as raw little-endian
float64, row-major N x N, to Ising2d_N{N}_alpha1.0.f64 beside this file;
build.py turns those into the Jmat{N}.h headers the drop-in executables
include (exact values, as hexadecimal floating literals).

The reference tree is taken from --reference, else from the environment
variable NQES_REFERENCE_DIR.
"""
import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# N of the reference's build list (code/build.sh:28), plus N = 50, the shape of
# the reference's published trapped-ion runs (data/energy/ion_N50_*).
SIZES = [8, 16, 32, 50, 64, 128]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("NQES_REFERENCE_DIR"))
    args = ap.parse_args()
    if not args.reference or not os.path.isdir(args.reference):
        sys.exit("give the reference tree with --reference or NQES_REFERENCE_DIR")
    import scipy.io as sio
    for n in SIZES:
        src = os.path.join(args.reference, "code", "Jmat", f"Ising2d_N{n}_alpha1.0.mat")
        J = np.asarray(sio.loadmat(src)["J"], dtype="<f8")
        if J.shape != (n, n):
            sys.exit(f"{src}: J is {J.shape}, expected ({n}, {n})")
        J.tofile(os.path.join(HERE, f"Ising2d_N{n}_alpha1.0.f64"))
        print(f"N={n}: max|J| = {np.abs(J).max():.6f}")


if __name__ == "__main__":
    main()
