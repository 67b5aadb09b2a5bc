"""Batched heat-conduction SIMP on the GPU against the same instances run one
by one through the single-problem path (and one against the oracle): per
instance compliance within 1e-6 at each of 8 iterations, densities of the last
iteration (mean abs < 1e-4), every solve at the FP64 true residual."""
import numpy as np
import pytest

from oracle import pyoracle as O

pytestmark = pytest.mark.gpu

INSTANCES = [dict(side=16, edge=0, patch_w=1, patch_i0=7, vf=0.4),
             dict(side=24, edge=1, patch_w=2, patch_i0=3, vf=0.35),
             dict(side=32, edge=2, patch_w=3, patch_i0=20, vf=0.5),
             dict(side=48, edge=3, patch_w=4, patch_i0=0, vf=0.3),
             dict(side=64, edge=0, patch_w=6, patch_i0=58, vf=0.45),
             dict(side=32, edge=1, patch_w=3, patch_i0=14, vf=0.42)]
ITERS = 8


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


@pytest.fixture(scope="module", params=[(256, 1), (256, 4), (512, 8)], ids=lambda p: f"{p[0]}x{p[1]}")
def batched(gpu, request):
    """threads per CTA x CTAs per instance (a thread-block cluster)"""
    from pansfem2_gb300.batch import HeatBatch
    threads, cluster = request.param
    with HeatBatch(INSTANCES, threads=threads, cluster=cluster) as B:
        B.begin(cg_eps=1e-10, cg_itmax=5000, warm_start=True)
        fs, res = [], []
        for _ in range(ITERS):
            B.step(1)
            r = B.results()
            fs.append(r["f"].copy())
            res.append(r["res"].copy())
            assert (r["conv"] == 1).all(), r
        rho = [B.fields(k)["rho"] for k in range(len(INSTANCES))]
        probs = [B.problem(k) for k in range(len(INSTANCES))]
    return np.array(fs), np.array(res), rho, probs


def test_batch_residuals(batched):
    _, res, _, _ = batched
    assert res.max() < 1e-10


@pytest.mark.parametrize("k", range(len(INSTANCES)))
def test_batch_matches_single_problem_path(gpu, batched, k):
    fs, _, rho, probs = batched
    with gpu.Problem(probs[k]) as P:
        P.setup_bc()
        P.simp_begin(solver="ir_mg_f32", cg_eps=1e-10)
        for it in range(ITERS):
            info = P.simp_step()
            assert abs(info["f"] - fs[it, k]) <= 1e-6 * abs(info["f"]), (k, it, info["f"], fs[it, k])
        # densities of the last iteration: the OC bisection takes its branch on the sign of the volume
        # constraint, and where g is within rounding of 0 the two summation orders may take different
        # branches (lambda then differs by the bisection tolerance); the compliance above is unaffected
        d = np.abs(P.fields()["rho"] - rho[k])
        assert d.mean() < 1e-4 and d.max() < 5e-2, (d.mean(), d.max())


def test_batch_matches_oracle(batched):
    fs, _, _, probs = batched
    ref = O.simp_run(dict(probs[0], cg_eps=1e-10), ITERS)
    assert np.max(np.abs(ref["f"] - fs[:, 0]) / np.abs(ref["f"])) < 1e-6
