"""GPU Heaviside projection filter (HeavisideFilter.h:16-98) with the samples'
beta continuation (beta *= 2 every 40 iterations, sample_optimize_density_oc.cpp:85-88):
the first iterations against the reference's own trajectory, and 44 iterations
(across the first doubling after k = 0 and the one at k = 40) against the oracle."""
import numpy as np
import pytest

from oracle import pyoracle as O
from pansfem2_gb300 import problems as PB
from tests.cases import CASES, load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


def test_heaviside_trajectory_matches_reference(gpu):
    name = "cantilever_12x6_heaviside"
    g, pr = load(name), CASES[name]()
    iters = int(g["iters"][0])
    ne = PB.counts(pr)[0]
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver="csr_jacobi_f64", cg_eps=1e-10)
        for k in range(iters):
            info = P.simp_step()
            fl = P.fields()
            assert abs(info["f"] - g["f"][k]) <= 1e-6 * abs(g["f"][k]), (k, info["f"], g["f"][k])
            assert np.max(np.abs(fl["rho"] - g["rho"].reshape(iters, ne)[k])) < 1e-6, k
            assert np.max(np.abs(fl["dfds"] - g["dfds"].reshape(iters, ne)[k])) <= 1e-6 * np.max(
                np.abs(g["dfds"].reshape(iters, ne)[k])), k


@pytest.mark.parametrize("solver", ["csr_jacobi_f64", "ir_mg_f32"])
def test_heaviside_continuation_matches_oracle(gpu, solver):
    pr = PB.cantilever_q4(12, 6, heaviside=1)
    iters = 44
    ref = O.simp_run(dict(pr, cg_eps=1e-10), iters)
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver=solver, cg_eps=1e-10)
        fs = [P.simp_step()["f"] for _ in range(iters)]
    fs = np.array(fs)
    rel = np.abs(fs - ref["f"]) / np.abs(ref["f"])
    assert rel.max() < 1e-5, (int(rel.argmax()), rel.max())
    # the doubling at k = 40 changes the projection: the compliance jumps there in both
    assert abs(ref["f"][40] - ref["f"][39]) > 1e-3 * abs(ref["f"][39])
