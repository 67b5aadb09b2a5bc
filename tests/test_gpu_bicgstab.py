"""GPU BiCGSTAB (CG.h:158-193) against the oracle's restatement (itself checked
against the reference's sol_bicgstab output in the golden fixtures) on the
reference's own assembled system, and on a nonsymmetric system against a
direct solve; through the generic C ABI and through a structured context."""
import numpy as np
import pytest

from oracle import pyoracle as O
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


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def test_bicgstab_on_the_reference_system(gpu):
    from pansfem2_gb300 import generic as G
    g = load("cantilever_12x6_oc")
    ip, ix, d, b = g["indptr"], g["indices"], g["data"], g["F0"]
    x_ref, it_ref = O.solve("bicgstab", ip, ix, d, b, eps=1e-10)
    x, info = G.csr_solve(ip, ix, d, b, solver="csr_bicgstab_f64", eps=1e-10)
    assert info["status"] == 0 and it_ref > 0
    assert abs(info["iterations"] - it_ref) <= max(2, it_ref // 20), (info["iterations"], it_ref)
    assert rel(x, x_ref) < 1e-8
    if "sol_bicgstab" in g:
        assert rel(x, g["sol_bicgstab"]) < 1e-8


def test_bicgstab_nonsymmetric(gpu):
    from pansfem2_gb300 import generic as G
    rng = np.random.default_rng(4)
    n = 3000
    rows, cols, vals = [], [], []
    for i in range(n):
        for j in (i - 7, i - 1, i, i + 1, i + 11):
            if 0 <= j < n:
                rows.append(i)
                cols.append(j)
                vals.append(6.0 if i == j else rng.uniform(-1.0, 1.0))
    A = np.zeros((n, n))
    A[rows, cols] = vals
    ip = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=n))]).astype(np.int32)
    order = np.lexsort((cols, rows))
    ix = np.array(cols)[order].astype(np.int32)
    d = np.array(vals)[order]
    b = rng.standard_normal(n)
    x, info = G.csr_solve(ip, ix, d, b, solver="csr_bicgstab_f64", eps=1e-12)
    assert info["status"] == 0
    assert rel(x, np.linalg.solve(A, b)) < 1e-10


def test_bicgstab_in_a_structured_context(gpu):
    pr = CASES["cantilever_12x6_oc"]()
    g = load("cantilever_12x6_oc")
    with gpu.Problem(pr) as P:
        P.setup_bc()
        from pansfem2_gb300 import problems as PB
        ne = PB.counts(pr)[0]
        rng = np.random.default_rng(2)
        rho = rng.uniform(0.1, 1.0, ne)   # a varied design: the filter does not matter for the solve
        E = pr["E1"] * rho ** pr["p"] + pr["E0"] * (1 - rho ** pr["p"])
        P.assemble(E)
        u_b, i_b = P.solve("csr_bicgstab_f64", eps=1e-10)
        u_c, i_c = P.solve("csr_jacobi_f64", eps=1e-10)
        assert i_b["status"] == 0 and i_b["rel_residual"] < 1e-9
        assert rel(u_b, u_c) < 1e-8
