"""GPU VTK output against the file the reference's own writer produced
(ExportToVTK.h, through the sample's call sequence) for iteration 0 of the
12x6 cantilever: identical structure (headers, counts, connectivity, cell
types), and the printed values of u, r and s equal to the 6 digits both
print, up to the solver tolerance on values near zero."""
import os

import numpy as np
import pytest

from tests.cases import CASES

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_cantilever_12x6_it0.vtk")


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


def sections(path):
    """Splits a legacy VTK file into (header line, [tokens]) sections."""
    out, cur = [], None
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if not t:
                continue
            if t[0][0].isalpha() or t[0].startswith("#"):
                cur = (line.strip(), [])
                out.append(cur)
            else:
                cur[1].extend(t)
    return out


def compare(path):
    ref, got = sections(GOLDEN), sections(path)
    assert [h for h, _ in got] == [h for h, _ in ref]
    for (h, a), (_, b) in zip(got, ref):
        assert len(a) == len(b), h
        if not a:
            continue
        fa, fb = np.array(a, float), np.array(b, float)
        if h.startswith(("CELLS", "CELL_TYPES")):
            assert np.array_equal(fa, fb), h
        else:
            tol = 1e-5 * np.abs(fb) + 1e-6 * max(np.abs(fb).max(), 1e-300)
            bad = np.abs(fa - fb) > tol
            assert not bad.any(), (h, np.argwhere(bad)[:5].ravel(), fa[bad][:5], fb[bad][:5])


@pytest.mark.parametrize("async_", [False, True])
def test_vtk_iteration0_matches_reference_writer(gpu, tmp_path, async_):
    pr = CASES["cantilever_12x6_oc"]()
    out = tmp_path / "result0.vtk"
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver="csr_jacobi_f64", cg_eps=1e-10)
        P.simp_step()
        P.export_vtk(out, async_=async_)
        P.simp_step()   # the next iteration runs while the file is written
        P.export_wait()
    compare(out)
