"""The oracle against the end states the reference's density-method samples ship with
(sample/optimize/Density_{OC,MMA,CONLIN}.vtk, extracted by tests/golden/make_sample_vtk.py):
run with the samples' own settings until IsConvergence, it stops at the same iteration and
its densities equal the file's to its 6 printed digits."""
import numpy as np
import pytest

from oracle import pyoracle as O
from tests.cases import load
from tests.samples import SAMPLES


@pytest.mark.parametrize("opt", sorted(SAMPLES))
def test_oracle_reproduces_the_sample_end_state(opt):
    g = load(f"sample_density_{opt}")
    make, _ = SAMPLES[opt]
    res = O.simp_run(make(), 500, fields=True, fast=True, stop_on_convergence=True)
    assert int(res["done"]) == int(g["iters"][0]), (res["done"], g["iters"])
    assert np.max(np.abs(res["rho"][int(res["done"]) - 1] - g["s"])) < 1e-6
