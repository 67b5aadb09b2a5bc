"""The device SIMP loop against the end states the reference's density-method samples ship
with (sample/optimize/Density_{OC,MMA,CONLIN}.vtk: the 60x40 cantilever with the Heaviside
filter and beta continuation, scale0 = 1e5, run until the optimiser's IsConvergence).  With
the reference's ScalingCG and with the multigrid FCG, each to 1e-10 as the samples solve, the
loop stops at the reference run's iteration and its densities equal the file's to its 6
printed digits."""
import numpy as np
import pytest

from tests.cases import load
from tests.samples import SAMPLES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


@pytest.mark.parametrize("solver", ["csr_jacobi_f64", "ir_mg_f32"])
@pytest.mark.parametrize("opt", sorted(SAMPLES))
def test_device_loop_reaches_the_sample_end_state(gpu, opt, solver):
    g = load(f"sample_density_{opt}")
    make, _ = SAMPLES[opt]
    with gpu.Problem(make()) as prob:
        prob.setup_bc()
        prob.simp_begin(solver=solver, cg_eps=1e-10)
        for k in range(500):
            info = prob.simp_step()
            assert info["solve"]["rel_residual"] < 1e-9, (k, info["solve"])
            if info["converged"]:
                break
        rho = prob.fields()["rho"]
    assert k + 1 == int(g["iters"][0]), (k + 1, g["iters"])
    assert np.max(np.abs(rho - g["s"])) < 1e-6
