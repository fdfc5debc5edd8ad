"""Generate the golden fixtures under tests/golden/ from the reference checkout.

The reference (ImmerseFlow++) ships result files produced by its own runs:
  results/uc.dat, results/vc.dat  -- ADsolver state after 20 steps, 52x52 grid
  results/p.dat                   -- Jacobi Laplace solve (PPESolver intent)
  results/final_results.dat       -- iBlank field
and the input surface (inputs/inputs.txt, inputs/xgrid.dat{,2}, ygrid.dat{,2}).

This script converts the Tecplot files to one compressed .npz (values as
printed, %f precision) plus the SHA-256 of each original file, and copies the
small input files verbatim.  It reads the reference only here, at fixture
generation time; the tests use the committed fixtures.

Usage:  python tests/golden/make_golden.py <reference checkout>
"""
import hashlib
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_tecplot(path):
    with open(path, "rb") as f:
        raw = f.read()
    lines = raw.decode().splitlines()
    zone = lines[2]
    ni = int(zone.split("I=")[1].split(",")[0])
    nj = int(zone.split("J=")[1].split(",")[0])
    vals = np.array([[float(t) for t in ln.split(",")] for ln in lines[3:3 + ni * nj]])
    x = vals[:ni, 0].copy()
    y = vals[::ni, 1].copy()
    q = vals[:, 2].reshape(nj, ni)  # q[j, i] = value at (x[i], y[j])
    return x, y, q, hashlib.sha256(raw).hexdigest()


def main(ref):
    out = {}
    digests = {}
    for name in ("uc", "vc", "p", "final_results"):
        x, y, q, h = read_tecplot(os.path.join(ref, "results", name + ".dat"))
        out["x"], out["y"] = x, y
        out[name] = q
        digests[name] = h
    np.savez_compressed(os.path.join(HERE, "results_52x52.npz"), **out)
    with open(os.path.join(HERE, "results_sha256.txt"), "w") as f:
        for k, v in digests.items():
            f.write(f"{k}.dat {v}\n")
    dst = os.path.join(HERE, "inputs")
    os.makedirs(dst, exist_ok=True)
    for fn in ("inputs.txt", "xgrid.dat", "ygrid.dat", "xgrid.dat2", "ygrid.dat2"):
        shutil.copyfile(os.path.join(ref, "inputs", fn), os.path.join(dst, fn))
    print("wrote", sorted(out), "and inputs/ into", HERE)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout>")
    main(sys.argv[1])
