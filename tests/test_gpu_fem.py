"""GPU explicit-mesh path (psf_fem_*) against the reference's own results on meshes with
permuted node ids, jittered coordinates, per-element moduli and prescribed nonzero values
(T3 and Q4 plane strain, Q4 heat, H8; tests/golden/fem_*.npz):

* numbering, CSR pattern, values and F bit-exact (the element matrices are computed with the
  reference's operation order, the entries summed in its element order);
* the reaction r = sum_e Ke_e u_e from the reference's own solution bit-exact;
* the solution of the GPU solve within 1e-8 relative of the reference's (a different
  summation order in the Krylov dot products).
"""
import numpy as np
import pytest

from tests.cases import load

pytestmark = pytest.mark.gpu

FEM_NAMES = ["fem_planestrain_sample", "fem_q4_jitter", "fem_q4_heat_jitter", "fem_t3_jitter", "fem_h8_jitter"]


@pytest.fixture(scope="module")
def fem():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pansfem2_gb300 import fem as F
    return F


def _mesh(fem, g):
    m = fem.FemMesh(int(g["kind"][0]), g["coords"], g["conn"])
    fx = g["fixed"]
    m.set_dirichlet(fx[:, 0].astype(int), fx[:, 1].astype(int), fx[:, 2])
    L = g["loads"]
    m.set_loads(L[:, 0].astype(int), L[:, 1].astype(int), L[:, 2])
    V, t = g["Vt"]
    m.assemble(g["E"], V, t)
    return m


@pytest.mark.parametrize("name", FEM_NAMES)
def test_system_bitexact(fem, name):
    g = load(name)
    with _mesh(fem, g) as m:
        n2g, ip, ix, d, F = m.system()
    for a, b in ((n2g, "n2g"), (ip, "indptr"), (ix, "indices"), (d, "data"), (F, "F")):
        assert np.array_equal(a, g[b]), b


@pytest.mark.parametrize("name", FEM_NAMES)
def test_reaction_bitexact_and_solution(fem, name):
    g = load(name)
    with _mesh(fem, g) as m:
        r = m.reaction(g["u"])
        u, info = m.solve("cg" if int(g["solver"][0]) == 4 else "scaling_cg", eps=1e-10)
        assert info["status"] == 0
    assert np.array_equal(r, g["r"])
    rel = np.max(np.abs(u - g["u"])) / np.max(np.abs(g["u"]))
    assert rel < 1e-8, rel
    # prescribed values are returned on the fixed dofs
    nd = len(u) // len(g["coords"])
    for n, d, v in g["fixed"]:
        assert u[int(n) * nd + int(d)] == v


def test_rejects_bad_connectivity(fem):
    g = load("fem_q4_jitter")
    conn = np.array(g["conn"])
    conn[0, 0] = len(g["coords"])   # out of range
    with pytest.raises(Exception):
        fem.FemMesh(int(g["kind"][0]), g["coords"], conn)
