"""The autotuner on the GPU: the PCG launch shape chosen by timing is set on the Problem, is
reused from the cache without timing again, and every shape solves to the same answer."""
import numpy as np
import pytest

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


def test_tune_pcg_sets_and_reuses_the_shape(gpu, tmp_path, monkeypatch):
    from pansfem2_gb300 import _lib, autotune
    monkeypatch.setenv("PSF_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_CACHE", {})
    pr = PB.mbb_q4(128, 64)
    with gpu.Problem(pr) as prob:
        prob.setup_bc()
        best, times = autotune.tune_pcg(prob, iters=50)
        assert len(times) >= 3 and best == min(((tuple(int(v) for v in k.split("x")), t) for k, t in times.items()),
                                               key=lambda kv: kv[1])[0]
        assert prob.launch_shape(_lib.PSF_KERNEL_PCG_CSR) == best
        sols = []
        for shape in ((1, 1024, 1), (4, 256, 4), (8, 512, 2), (16, 1024, 1), best):
            prob.set_launch_shape(_lib.PSF_KERNEL_PCG_CSR, *shape)
            u, info = prob.solve("csr_jacobi_f64", eps=1e-10)
            assert info["status"] == 0
            sols.append(u)
        for u in sols[1:]:
            assert np.max(np.abs(u - sols[0])) <= 1e-8 * np.max(np.abs(sols[0]))
    # cached: a second tuning of the same problem times nothing (its solves would fail here)
    with gpu.Problem(pr) as prob:
        prob.setup_bc()

        def no_solve(*a, **k):
            raise AssertionError("timed again")

        monkeypatch.setattr(prob, "solve", no_solve)
        best2, _ = autotune.tune_pcg(prob, iters=50)
        assert best2 == best and prob.launch_shape(_lib.PSF_KERNEL_PCG_CSR) == best
