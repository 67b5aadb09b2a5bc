"""3D H8 cantilever (the linear-elastic workload): the mixed-precision multigrid
FCG against the oracle on a grid that coarsens, a SIMP trajectory, and the
full 128x64x64 grid (1,635,075 dofs) against the FP64 matrix-free Jacobi PCG."""
import numpy as np
import pytest

from oracle import pyoracle as O
from pansfem2_gb300 import problems as PB

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def test_h8_multigrid_trajectory_matches_oracle(gpu):
    pr = PB.cantilever_h8(16, 8, 8)
    iters = 5
    ref = O.simp_run(dict(pr, cg_eps=1e-10), iters, fields=True)
    ne = PB.counts(pr)[0]
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver="ir_mg_f32", cg_eps=1e-10)
        for k in range(iters):
            info = P.simp_step()
            assert info["solve"]["rel_residual"] < 1e-9, (k, info["solve"])
            fl = P.fields()
            assert abs(info["f"] - ref["f"][k]) <= 1e-6 * abs(ref["f"][k]), (k, info["f"], ref["f"][k])
            assert np.max(np.abs(fl["rho"] - ref["rho"].reshape(iters, ne)[k])) < 1e-6, k


def test_h8_full_size_multigrid_vs_fp64(gpu):
    pr = PB.cantilever_h8(128, 64, 64)
    ne = PB.counts(pr)[0]
    rng = np.random.default_rng(3)
    E = 1e-9 + (1 - 1e-9) * rng.uniform(0.2, 1.0, ne) ** 3
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.assemble(E)
        u_mg, i_mg = P.solve("ir_mg_f32", itmax=5000, eps=1e-8)
        assert i_mg["status"] == 0 and i_mg["rel_residual"] < 1e-8, i_mg
        u_64, i_64 = P.solve("ebe_jacobi_f64", itmax=200000, eps=1e-8)
        assert i_64["status"] == 0 and i_64["rel_residual"] < 1.5e-8, i_64
        assert rel(u_mg, u_64) < 1e-5
        assert i_mg["iterations"] * 10 < i_64["iterations"]
