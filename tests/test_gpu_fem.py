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


def _oracle_system(kind, coords, conn, E, V, t, fixed, loads, body=None, edges=None, traction=None):
    from oracle import pyoracle as O
    nd = {0: 2, 1: 1, 2: 3, 3: 2}[kind]
    nn = len(coords)
    fx = np.zeros(nn * nd, np.uint8)
    uf = np.zeros(nn * nd)
    for n, d, v in fixed:
        fx[int(n) * nd + int(d)] = 1
        uf[int(n) * nd + int(d)] = v
    n2g, N = O.renumber(nn, nd, fx)
    ip, ix, dat, F = O.assemble(kind, conn, coords, E, n2g, N, V, t, ufixed=uf, body=body)
    F = O.neumann(F, loads[:, 0].astype(int), loads[:, 1].astype(int), loads[:, 2], nd, n2g)
    if edges is not None and len(edges):
        F = O.edge_loads(F, edges, coords, traction, t, n2g)
    return n2g, ip, ix, dat, F


def _gpu_system(fem, kind, coords, conn, E, V, t, fixed, loads, body=None, edges=None, traction=None):
    with fem.FemMesh(kind, coords, conn) as m:
        m.set_dirichlet(fixed[:, 0].astype(int), fixed[:, 1].astype(int), fixed[:, 2])
        m.set_loads(loads[:, 0].astype(int), loads[:, 1].astype(int), loads[:, 2])
        if body is not None:
            m.set_body_force(*body)
        if edges is not None and len(edges):
            m.set_edge_loads(edges, *traction)
        m.assemble(E, V, t)
        return m.system()


def test_midsize_q4_mesh_against_the_oracle(fem):
    """256x128 jittered Q4 mesh with permuted node ids (66k dofs, 1.2M stored entries), body
    force, top-edge tractions and a point load: the whole system bit-exact with the oracle."""
    from pansfem2_gb300 import problems as PB
    m = PB.jittered_q4_mesh(256, 128, seed=7)
    args = (0, m["coords"], m["conn"], m["E"], m["V"], m["t"], m["fixed"], m["loads"], m["body"], m["edges"],
            m["traction"])
    for a, b, name in zip(_gpu_system(fem, *args), _oracle_system(*args), ("n2g", "indptr", "indices", "data", "F")):
        assert np.array_equal(a, b), name


def test_midsize_h8_mesh_against_the_oracle(fem):
    """12x10x8 jittered H8 mesh with permuted node ids, per-element moduli, a clamped face with
    a prescribed nonzero value and point loads: bit-exact with the oracle (rows of up to 81
    columns, nodes with 26 neighbours)."""
    rng = np.random.default_rng(11)
    nx, ny, nz = 12, 10, 8
    nn = (nx + 1) * (ny + 1) * (nz + 1)
    perm = rng.permutation(nn)
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    grid = np.stack([i, j, k], -1).reshape(-1, 3).astype(float)
    coords = np.empty_like(grid)
    coords[perm] = grid + rng.uniform(-0.2, 0.2, grid.shape)
    nid = lambda a, b, c: perm[(a * (ny + 1) + b) * (nz + 1) + c]  # noqa: E731
    I, J, K = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    conn = np.stack([nid(I, J, K), nid(I + 1, J, K), nid(I + 1, J + 1, K), nid(I, J + 1, K),
                     nid(I, J, K + 1), nid(I + 1, J, K + 1), nid(I + 1, J + 1, K + 1), nid(I, J + 1, K + 1)],
                    -1).reshape(-1, 8).astype(np.int32)
    E = rng.uniform(0.2, 1.0, len(conn))
    face = [nid(0, b, c) for b in range(ny + 1) for c in range(nz + 1)]
    fixed = np.array([(n, d, 0.0) for n in face for d in range(3)] + [(nid(nx, 0, 0), 2, 0.01)], float)
    loads = np.array([(nid(nx, b, nz), 2, -0.1) for b in range(ny + 1)], float)
    args = (2, coords, conn, E, 0.3, 1.0, fixed, loads)
    for a, b, name in zip(_gpu_system(fem, *args), _oracle_system(*args), ("n2g", "indptr", "indices", "data", "F")):
        assert np.array_equal(a, b), name


def test_kernel_launch_counter(fem):
    """psf_kernel_launches counts every launch: the first assembly of an H8 mesh runs the element
    kernel, the pattern count, a three-kernel scan and the values kernel; a second one reuses
    the pattern."""
    from pansfem2_gb300 import _lib
    g = load("fem_h8_jitter")
    with _mesh(fem, g) as m:
        V, t = g["Vt"]
        l0 = _lib.kernel_launches()
        m.assemble(g["E"], V, t)
        assert _lib.kernel_launches() - l0 == 2
    with fem.FemMesh(int(g["kind"][0]), g["coords"], g["conn"]) as m:
        fx = g["fixed"]
        m.set_dirichlet(fx[:, 0].astype(int), fx[:, 1].astype(int), fx[:, 2])
        l0 = _lib.kernel_launches()
        m.assemble(g["E"], *g["Vt"])
        assert _lib.kernel_launches() - l0 == 6
