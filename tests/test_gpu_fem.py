"""GPU explicit-mesh path (psf_fem_*) against the reference's own results on meshes with
permuted node ids, jittered coordinates, per-element moduli and prescribed nonzero values
(T3 and Q4 plane strain, Q4 heat, H8; tests/golden/fem_*.npz):

* numbering, CSR pattern, values and F bit-exact (the element matrices are computed with the
  reference's operation order, the entries summed in its element order);
* the reaction r = sum_e Ke_e u_e from the reference's own solution bit-exact;
* the solution of the GPU solve within 1e-8 relative of the reference's (a different
  summation order in the Krylov dot products);
* the reference's H8 sample (sample/solid/sample_linear.cpp), its mesh and conditions written
  as CSV files and read back by pansfem2_gb300.csvio, and by the C++ mirror of the API
  (tests/cpp/sample_solid_gpu.cpp): the solution agrees with the reference's and with the six
  digits of its committed result_linear.vtk.
"""
import os
import subprocess

import numpy as np
import pytest

from tests.cases import load

pytestmark = pytest.mark.gpu

FEM_NAMES = ["fem_planestrain_sample", "fem_q4_jitter", "fem_q4_heat_jitter", "fem_t3_jitter", "fem_h8_jitter",
             "fem_solid_sample"]
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


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
    if not np.isnan(g["body"]).any():
        m.set_body_force(*g["body"])
    if len(g["edges"]):
        m.set_edge_loads(g["edges"], *g["traction"])
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


def _write_csv(g, path):
    """The golden mesh and conditions as the reference's CSV files (sample/solid layout)."""
    os.makedirs(path, exist_ok=True)
    nd = {0: 2, 1: 1, 2: 3, 3: 2}[int(g["kind"][0])]
    with open(os.path.join(path, "Node.csv"), "w") as fh:
        fh.write("ID," + ",".join(f"x{d}" for d in range(g["coords"].shape[1])) + "\n")
        for i, x in enumerate(g["coords"]):
            fh.write(f"{i}," + ",".join(repr(float(v)) for v in x) + "\n")
    with open(os.path.join(path, "Element.csv"), "w") as fh:
        fh.write("ID," + ",".join(f"n{q}" for q in range(g["conn"].shape[1])) + "\n")
        for e, el in enumerate(g["conn"]):
            fh.write(f"{e}," + ",".join(str(int(n)) for n in el) + "\n")
    for fname, rows in (("Dirichlet.csv", g["fixed"]), ("Neumann.csv", g["loads"])):
        nodes = list(dict.fromkeys(int(n) for n in rows[:, 0]))
        with open(os.path.join(path, fname), "w") as fh:
            fh.write("idn," + ",".join(f"d{d}" for d in range(nd)) + "\n")
            for n in nodes:
                vals = ["free"] * nd
                for m, d, v in rows:
                    if int(m) == n:
                        vals[int(d)] = repr(float(v))
                fh.write(f"{n}," + ",".join(vals) + "\n")


def _check_solid(u, g):
    rel = np.max(np.abs(u - g["u"])) / np.max(np.abs(g["u"]))
    assert rel < 1e-8, rel
    # result_linear.vtk holds 6 significant digits of the reference's solution
    vtk = g["vtk_u"].reshape(-1)
    assert np.all(np.abs(u - vtk) <= 5e-6 * np.abs(vtk) + 1e-12), np.max(np.abs(u - vtk))


def test_solid_sample_from_csv(fem, tmp_path):
    from pansfem2_gb300 import csvio
    g = load("fem_solid_sample")
    d = str(tmp_path / "solid")
    _write_csv(g, d)
    x = csvio.import_nodes_from_csv(os.path.join(d, "Node.csv"))
    el = csvio.import_elements_from_csv(os.path.join(d, "Element.csv"))
    fixed = csvio.conditions_arrays(csvio.import_dirichlet_from_csv(os.path.join(d, "Dirichlet.csv")))
    loads = csvio.conditions_arrays(csvio.import_neumann_from_csv(os.path.join(d, "Neumann.csv")))
    assert np.array_equal(x.reshape(-1), g["read_coords"]) and np.array_equal(el.reshape(-1), g["read_conn"])
    with fem.FemMesh(2, x, el) as m:
        m.set_dirichlet(*fixed)
        m.set_loads(*loads)
        m.assemble(np.full(len(el), 210000.0), 0.3, 1.0)
        n2g, ip, ix, dat, F = m.system()
        u, info = m.solve("scaling_cg", eps=1e-10)
    for a, b in ((n2g, "n2g"), (ip, "indptr"), (ix, "indices"), (dat, "data"), (F, "F")):
        assert np.array_equal(a, g[b]), b
    assert info["status"] == 0
    _check_solid(u, g)


def test_solid_sample_cpp(fem, tmp_path):
    from pansfem2_gb300 import _lib
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "sample_solid_gpu")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "sample_solid_gpu.cpp"), "-o", exe,
                    "-L", libdir, "-lpansfem2_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    g = load("fem_solid_sample")
    d = str(tmp_path / "solid")
    _write_csv(g, d)
    out = subprocess.run([exe, d], check=True, capture_output=True, text=True).stdout
    rows = [l.split() for l in out.splitlines() if l.startswith("u ")]
    u = np.array([[float(v) for v in r[2:5]] for r in rows]).reshape(-1)
    assert int(out.split()[1]) == len(g["F"])
    _check_solid(u, g)
