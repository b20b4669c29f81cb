"""Fixtures from the reference's own published data (run with the reference tree).

    python tests/golden/make_ref_fixtures.py [--reference DIR]

(DIR defaults to the environment variable NQES_REFERENCE_DIR.)

Writes tests/golden/ref_trained_N50M150K2.npz and ref_energy_tails.json:

* the trained complex weights a (K x N), b (K x M), w (K x N x M) of
  data/rbm-weights/ionh0.595train{1.2,2.2}N50M150K2.mat, read with
  scipy.io.loadmat (the layout code/rbm.cc:272-385 loads);
* for each, the per-site energies the reference printed over the last 20 SR
  steps of the run that dumped those weights (data/energy/
  ion_N50_M150_K2_h0.595_c128_m200-{1,2}: the second command of each log has
  --load-rbm ionh0.595train{1,2}N50M150K2.mat --dump-rbm ionh0.595train{1,2}.2),
  with the file and line numbers they come from, and the run's flags.

These runs use the reference's compiled-in couplings
code/Jmat/Ising2d_N50_alpha1.0.mat (nqes-trapped-ion_gb300/cli/jmat/
Ising2d_N50_alpha1.0.f64 holds the same values), h = 0.595, 128 chains x 200
samples, burn-in 64.
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RUNS = [("ionh0.595train1.2N50M150K2.mat", "ion_N50_M150_K2_h0.595_c128_m200-1", "ionh0.595train1.2"),
        ("ionh0.595train2.2N50M150K2.mat", "ion_N50_M150_K2_h0.595_c128_m200-2", "ionh0.595train2.2")]
TAIL = 20


def energy_tail(path, dump_prefix):
    """(first line, last line, energies) of the last TAIL energy lines of the
    command that ends with --dump-rbm dump_prefix (1-based line numbers)."""
    with open(path) as f:
        lines = f.read().split("\n")
    start = next(i for i, ln in enumerate(lines) if ln.rstrip().endswith("--dump-rbm " + dump_prefix))
    cmd = lines[start]
    rows = []
    for i in range(start + 1, len(lines)):
        if lines[i].startswith("Program exited"):
            break
        try:
            vals = [float(x) for x in lines[i].split()]
        except ValueError:
            continue
        if vals:
            rows.append((i + 1, vals))
    tail = rows[-TAIL:]
    return cmd, tail[0][0], tail[-1][0], [v for _, v in tail]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("NQES_REFERENCE_DIR"))
    args = ap.parse_args()
    if not args.reference or not os.path.isdir(args.reference):
        sys.exit("give the reference tree with --reference or NQES_REFERENCE_DIR")
    import scipy.io as sio
    arrays, tails = {}, []
    for t, (wfile, log, prefix) in enumerate(RUNS):
        m = sio.loadmat(os.path.join(args.reference, "data", "rbm-weights", wfile))
        for name in ("a", "b", "w"):
            arrays[f"{name}{t}"] = np.ascontiguousarray(m[name], dtype=np.complex128)
        cmd, l0, l1, e = energy_tail(os.path.join(args.reference, "data", "energy", log), prefix)
        tails.append({"weights": f"data/rbm-weights/{wfile}", "npz_index": t, "log": f"data/energy/{log}",
                      "lines": [l0, l1], "command": cmd.strip(), "energies_per_site": e})
    np.savez_compressed(os.path.join(HERE, "ref_trained_N50M150K2.npz"), **arrays)
    with open(os.path.join(HERE, "ref_energy_tails.json"), "w") as f:
        json.dump({"N": 50, "M": 150, "K": 2, "h": 0.595, "chains": 128, "samples_per_chain": 200, "burn_in": 64,
                   "jmat": "code/Jmat/Ising2d_N50_alpha1.0.mat", "runs": tails}, f, indent=1)
    for r in tails:
        e = np.array(r["energies_per_site"])
        print(r["log"], r["lines"], e.mean(0), e.std(0, ddof=1))


if __name__ == "__main__":
    main()
