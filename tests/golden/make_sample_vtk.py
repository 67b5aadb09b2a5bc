"""Extracts the end states the reference's SIMP samples ship with into fixtures.

The reference commits the last density field of each of its density-method samples
(sample/optimize/Density_OC.vtk, Density_MMA.vtk, Density_CONLIN.vtk: the 60x40
cantilever with the Heaviside filter and beta continuation, run until the optimiser's
IsConvergence).  This script reads the cell scalars "s" of those files (the filtered
densities of the last iteration, printed to 6 digits) and the run length at which the
oracle reproduces them, and stores both as tests/golden/sample_density_<opt>.npz.
Needs the reference source tree, so it runs only where that tree exists; the
fixtures it writes are committed and used everywhere else.

    python tests/golden/make_sample_vtk.py [path-to-PANSFEM2]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import build as obuild  # noqa: E402
from oracle import pyoracle as O  # noqa: E402
from tests.samples import SAMPLES  # noqa: E402


def read_cell_scalars(path, name):
    with open(path) as fh:
        lines = fh.read().split("\n")
    n = None
    for i, line in enumerate(lines):
        if line.startswith("CELL_DATA"):
            n = int(line.split()[1])
        if line.startswith("SCALARS " + name):
            vals, j = [], i + 2   # the next line is LOOKUP_TABLE
            while len(vals) < n:
                vals += [float(v) for v in lines[j].split()]
                j += 1
            return np.array(vals)
    raise ValueError(f"{path}: no cell scalars {name}")


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else obuild.REFERENCE_ROOT
    obuild.build()
    O.set_threads(os.cpu_count() or 1, fast=True)
    for opt, (make, vtk) in SAMPLES.items():
        s_vtk = read_cell_scalars(os.path.join(ref_root, "sample", "optimize", vtk), "s")
        res = O.simp_run(make(), 500, fields=True, fast=True, stop_on_convergence=True)
        iters = int(res["done"])
        err = float(np.max(np.abs(res["rho"][iters - 1] - s_vtk)))
        assert err < 1e-6, (opt, iters, err)
        np.savez_compressed(os.path.join(HERE, f"sample_density_{opt}.npz"), s=s_vtk, iters=np.array([iters]))
        print(f"sample_density_{opt}.npz: {vtk}, {iters} iterations, oracle within {err:.1e}")


if __name__ == "__main__":
    main()
