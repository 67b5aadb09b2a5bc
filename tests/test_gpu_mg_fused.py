"""The multigrid FCG with its grid levels fused (one grid phase per down-leg and per up-leg,
the intermediate sweeps recomputed on each block's grown tile) against the three-phase
levels: the V-cycle does the same arithmetic on every node, so one cycle agrees bit for bit
and whole solves to rounding, on even and odd grids, for the three element kinds.  PSF_MG_FUSE selects: 0 no level
fused, 1 the default choice, 2 every grid level."""
import os

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


CASES = {
    "mbb_256x128": lambda: PB.mbb_q4(256, 128),
    "mbb_odd_183x77": lambda: PB.mbb_q4(183, 77),
    "cantilever_60x30": lambda: PB.cantilever_q4(60, 30),
    "heatsink_96": lambda: PB.heatsink_q4(96, 96),
    "cantilever_h8_24x12x12": lambda: PB.cantilever_h8(24, 12, 12),
}


def with_mode(mode, fn):
    old = os.environ.get("PSF_MG_FUSE")
    os.environ["PSF_MG_FUSE"] = str(mode)
    try:
        return fn()
    finally:
        if old is None:
            del os.environ["PSF_MG_FUSE"]
        else:
            os.environ["PSF_MG_FUSE"] = old


def design(pr):
    ne = PB.counts(pr)[0]
    rng = np.random.default_rng(5)
    rho = rng.uniform(0.05, 1.0, ne)   # a ragged design: SIMP contrast up to 1e-4 in the moduli
    return pr["E1"] * rho ** pr["p"] + pr["E0"] * (1.0 - rho ** pr["p"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_fused_cycle_is_bit_identical(gpu, name):
    """One V-cycle (psf_mg_precondition) under every fusion mode: the same bits."""
    pr = CASES[name]()
    E = design(pr)
    with gpu.Problem(pr) as prob:
        prob.setup_bc()
        prob.assemble(E)
        r = np.random.default_rng(1).standard_normal(prob.nfree)
        z = {m: with_mode(m, lambda: prob.mg_precondition(r)) for m in (0, 1, 2, 3)}
    assert np.all(np.isfinite(z[0])) and np.linalg.norm(z[0]) > 0
    for m in (1, 2, 3):
        assert np.array_equal(z[m], z[0]), (m, float(np.max(np.abs(z[m] - z[0]))))


@pytest.mark.parametrize("name", sorted(CASES))
def test_fused_solves_agree(gpu, name):
    """Whole FCG solves: the cycle is identical, the dot products sum the same terms in the
    tile order instead of the grid-stride order, so iterates agree to rounding."""
    pr = CASES[name]()
    E = design(pr)

    def run():
        with gpu.Problem(pr) as prob:
            prob.setup_bc()
            prob.assemble(E)
            return prob.solve("ir_mg_f32", eps=1e-9)

    runs = {m: with_mode(m, run) for m in (0, 1, 2)}
    u0, i0 = runs[0]
    assert i0["status"] == 0 and i0["rel_residual"] < 1e-9, i0
    for m in (1, 2):
        u, info = runs[m]
        assert info["status"] == 0 and info["rel_residual"] < 1e-9, info
        assert abs(info["iterations"] - i0["iterations"]) <= max(2, i0["iterations"] // 10), \
            (m, info["iterations"], i0["iterations"])
        assert np.max(np.abs(u - u0)) <= 1e-8 * np.max(np.abs(u0)), m
