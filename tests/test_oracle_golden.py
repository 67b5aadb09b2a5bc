"""Pins the C oracle to the PANSFEM2 reference: every golden fixture was
produced by the reference itself (tests/golden/make_golden.py); the oracle
must reproduce it bit for bit (same operation order, -ffp-contract=off)."""
import numpy as np
import pytest

from oracle import pyoracle as O
from pansfem2_gb300 import problems as PB
from tests.cases import CASES, load


def geometry(pr):
    if pr["kind"] == PB.H8_SOLID:
        coords = O.h8_nodes(pr["lx"], pr["ly"], pr["lz"], pr["nx"], pr["ny"], pr["nz"])
        conn = O.h8_elements(pr["nx"], pr["ny"], pr["nz"])
        return coords, conn, 3
    return O.q4_nodes(pr["lx"], pr["ly"], pr["nx"], pr["ny"]), O.q4_elements(pr["nx"], pr["ny"]), 2


def same(a, b):
    a, b = np.asarray(a), np.asarray(b).reshape(np.asarray(a).shape)
    return np.array_equal(a, b)


@pytest.mark.parametrize("name", sorted(CASES))
def test_bc_lists_match_generate_fixedlist(name):
    g, pr = load(name), CASES[name]()
    for k in ("fix_node", "fix_dof", "load_node", "load_dof", "load_val"):
        assert same(g[k], pr[k]), k


@pytest.mark.parametrize("name", sorted(CASES))
def test_numbering_pattern_values_bitexact(name):
    g, pr = load(name), CASES[name]()
    if "indptr" not in g:
        pytest.skip("fixture keeps no CSR")
    coords, conn, dim = geometry(pr)
    ne, nn, nd = PB.counts(pr)
    n2g, N = O.renumber(nn, nd, PB.fixed_mask(pr))
    assert same(g["n2g"], n2g)
    rho0 = O.density_filter(*O.neighbors(O.centroids(conn, coords, dim), pr["R"]), np.full(ne, pr["rho0"]))
    E = pr["E1"] * np.power(rho0, pr["p"]) + pr["E0"] * (1.0 - np.power(rho0, pr["p"]))
    ipr, ind, dat, F = O.assemble(pr["kind"], conn, coords, E, n2g, N, pr["V"], pr["t"])
    F = O.neumann(F, pr["load_node"], pr["load_dof"], pr["load_val"], nd, n2g)
    assert same(g["indptr"], ipr) and same(g["indices"], ind)
    assert same(g["data"], dat) and same(g["F0"], F)
    x, it = O.solve("scaling_cg", ipr, ind, dat, F, eps=pr["cg_eps"])
    assert it > 0 and same(g["result0"], x)


@pytest.mark.parametrize("name", sorted(CASES))
def test_element_matrix_and_filter_bitexact(name):
    g, pr = load(name), CASES[name]()
    coords, conn, dim = geometry(pr)
    if "Ke0" in g:
        assert same(g["Ke0"], O.ke(pr["kind"], coords[conn[0]], 1.0, pr["V"], pr["t"]))
    if "Ke_last_E037" in g:
        assert same(g["Ke_last_E037"], O.ke(pr["kind"], coords[conn[-1]], 0.37, pr["V"], pr["t"]))
    cg = O.centroids(conn, coords, dim)
    if "centroids" in g:
        assert same(g["centroids"], cg)
    grid = [pr["nx"], pr["ny"], pr["nz"] if pr["kind"] == PB.H8_SOLID else 0]
    for gr in (None, grid):  # all-pairs and windowed search give the same lists
        ptr, idx, w = O.neighbors(cg, pr["R"], grid=gr)
        assert same(g["nb_ptr"], ptr) and same(g["nb_idx"], idx) and same(g["nb_w"], w)


@pytest.mark.parametrize("name", sorted(CASES))
def test_simp_trajectory_bitexact(name):
    g, pr = load(name), CASES[name]()
    iters = int(g["iters"][0])
    res = O.simp_run(pr, iters, fields=True)
    assert res["done"] == iters
    for k in ("f", "g", "rho", "dfdrho", "dfds", "s_after", "u"):
        if k in g:
            assert same(g[k], res[k]), k


def test_solver_suite_bitexact():
    """CG, BiCGSTAB, BiCGSTAB2, ScalingBiCGSTAB, ILU0 (factor + apply), ILU0CG and ILU0BiCGSTAB of CG.h."""
    g, pr = load("cantilever_12x6_oc"), CASES["cantilever_12x6_oc"]()
    ipr, ind, dat, F = g["indptr"], g["indices"], g["data"], g["F0"]
    for kind, key in (("cg", "sol_cg"), ("bicgstab", "sol_bicgstab"), ("bicgstab2", "sol_bicgstab2"),
                      ("ilu0_cg", "sol_ilu0cg"), ("scaling_bicgstab", "sol_scalingbicgstab"),
                      ("ilu0_bicgstab", "sol_ilu0bicgstab")):
        x, it = O.solve(kind, ipr, ind, dat, F, eps=1e-10)
        assert same(g[key], x), kind
    mi, mj, md = O.ilu0(ipr, ind, dat)
    assert same(g["ilu_indptr"], mi) and same(g["ilu_indices"], mj) and same(g["ilu_data"], md)


def _fmt(v):
    return "%g" % v


def _mma_trace(n, m, x0, a0, a, c, d, xmin, xmax, params, iters, fg):
    """Drives the oracle MMA the way the reference's test mains do and prints
    the same lines (C++ ostream default precision == %g)."""
    mma = O.MMA(n, m, a0, a, c, d, xmin, xmax)
    mma.set_parameters(*params)
    s = np.array(x0, float)
    out = ""
    for k in range(iters):
        f, df, g, dg, labels = fg(s)
        out += "\nk = %d\t" % k
        out += labels[0] + ":\t" + _fmt(f) + "\t"
        for lab, gi in zip(labels[1:], g):
            out += lab + ":\t" + _fmt(gi) + "\t"
        for si in s:
            out += "\t" + _fmt(si)
        if mma.is_convergence(f):
            out += "\n--------------------Optimized--------------------\n"
            break
        s, _ = mma.update(s, f, df, g, dg)
    return out


def test_reference_test_MMA():
    """src/Optimize/Solver/test_MMA.cpp (n=5, m=1: the SIMP branch n > m)."""
    C1, C2 = 0.0624, 1.0
    coef = np.array([61.0, 37.0, 19.0, 7.0, 1.0])

    def fg(s):
        f = C1 * (s[0] + s[1] + s[2] + s[3] + s[4])
        g = 61.0 * s[0] ** -3.0 + 37.0 * s[1] ** -3.0 + 19.0 * s[2] ** -3.0 + 7.0 * s[3] ** -3.0 + 1.0 * s[4] ** -3.0 - C2
        dg = [-3.0 * coef[j] * s[j] ** -4.0 for j in range(5)]
        return f, [C1] * 5, [g], [dg], ["Objective", "Constraints"]

    got = _mma_trace(5, 1, [5.0] * 5, 1.0, [0.0], [1000.0], [1.0], [1.0] * 5, [10.0] * 5,
                     (1e-5, 0.1, 0.5, 0.5, 0.7, 1.2, 1e-5), 10, fg)
    assert got == open(O.os.path.join(O.os.path.dirname(__file__), "..", "tests", "golden", "ref_test_MMA.txt")).read()


def test_reference_test_MMA_3():
    """src/Optimize/Solver/test_MMA_3.cpp (n=2, m=2: the n <= m branch)."""
    C1, C2 = 1.0, 0.124

    def fg(s):
        q = np.sqrt(1.0 + s[1] ** 2.0)
        f = C1 * s[0] * q
        df = [C1 * q, C1 * s[0] * s[1] / q]
        g0 = C2 * q * (8.0 * s[0] ** -1.0 + 1.0 * s[0] ** -1.0 * s[1] ** -1.0) - 1.0
        g1 = C2 * q * (8.0 * s[0] ** -1.0 - 1.0 * s[0] ** -1.0 * s[1] ** -1.0) - 1.0
        dg0 = [C2 * q * (-8.0 * s[0] ** -2.0 - 1.0 * s[0] ** -2.0 * s[1] ** -1.0),
               C2 * s[1] / q * (8.0 * s[0] ** -1.0 + 1.0 * s[0] ** -1.0 * s[1] ** -1.0)
               + C2 * q * (-1.0 * s[0] ** -1.0 * s[1] ** -2.0)]
        dg1 = [C2 * q * (-8.0 * s[0] ** -2.0 + 1.0 * s[0] ** -2.0 * s[1] ** -1.0),
               C2 * s[1] / q * (8.0 * s[0] ** -1.0 - 1.0 * s[0] ** -1.0 * s[1] ** -1.0)
               + C2 * q * (1.0 * s[0] ** -1.0 * s[1] ** -2.0)]
        return f, df, [g0, g1], [dg0, dg1], ["Objective", "Constraints0", "Constraints1"]

    got = _mma_trace(2, 2, [1.5, 0.5], 1.0, [0.0, 0.0], [1000.0, 1000.0], [1.0, 1.0], [0.2, 0.1],
                     [4.0, 1.6], (1e-5, 0.1, 0.5, 0.5, 0.7, 1.2, 1e-5), 100, fg)
    ref = open(O.os.path.join(O.os.path.dirname(__file__), "..", "tests", "golden", "ref_test_MMA_3.txt")).read()
    assert got == ref


def test_reference_test_MMA_TOY2():
    """src/Optimize/Solver/test_MMA_TOY2.cpp (n=3, m=2)."""
    def fg(s):
        f = s[0] ** 2.0 + s[1] ** 2.0 + s[2] ** 2.0
        g0 = (s[0] - 5.0) ** 2.0 + (s[1] - 2.0) ** 2.0 + (s[2] - 1.0) ** 2.0 - 9.0
        g1 = (s[0] - 3.0) ** 2.0 + (s[1] - 4.0) ** 2.0 + (s[2] - 3.0) ** 2.0 - 9.0
        return (f, [2.0 * s[0], 2.0 * s[1], 2.0 * s[2]], [g0, g1],
                [[2.0 * (s[0] - 5.0), 2.0 * (s[1] - 2.0), 2.0 * (s[2] - 1.0)],
                 [2.0 * (s[0] - 3.0), 2.0 * (s[1] - 4.0), 2.0 * (s[2] - 3.0)]], ["f", "g1", "g2"])

    got = _mma_trace(3, 2, [4.0, 3.0, 2.0], 1.0, [0.0, 0.0], [1000.0, 1000.0], [1.0, 1.0], [0.0] * 3,
                     [5.0] * 3, (1e-5, 0.1, 0.5, 0.5, 0.7, 1.2, 1e-5), 10, fg)
    ref = open(O.os.path.join(O.os.path.dirname(__file__), "..", "tests", "golden", "ref_test_MMA_TOY2.txt")).read()
    assert got == ref


@pytest.mark.parametrize("problem", ["mma", "mma3", "toy2"])
def test_conlin_steps_bitexact(problem):
    """CONLIN::UpdateVariables (CONLIN.h:91-365) replayed one step at a time on the
    reference's own iterates for the optimiser test problems: n > m (mma: n=5, m=1)
    and both n <= m reductions (mma3: n=2, m=2; toy2: n=3, m=2)."""
    d = load("conlin_" + problem)
    n, m = (int(v) for v in d["nm"])
    K = len(d["f"])
    assert K >= 5
    o = O.CONLIN(n, m, 1.0, [0.0] * m, [1000.0] * m, [1.0] * m, d["xmin"], d["xmax"])
    o.set_parameters(0.5, 1e-5)
    for k in range(K):
        x, newton = o.update(d["xin"][k * n:(k + 1) * n], d["f"][k], d["df"][k * n:(k + 1) * n],
                             d["g"][k * m:(k + 1) * m], d["dg"][k * m * n:(k + 1) * m * n])
        assert newton > 0
        assert same(d["xout"][k * n:(k + 1) * n], x), k


def test_reference_test_CG():
    """src/LinearAlgebra/Solvers/test_CG.cpp: 4x4 non-symmetric A built with
    CSR::set, b = A*1, BiCGSTAB2 -> prints 1 four times."""
    A = [[1.0, 1.0, 0.0, 3.0], [2.0, 1.0, -1.0, 1.0], [3.0, -1.0, -1.0, 2.0], [-1.0, 2.0, 3.0, -1.0]]
    indptr = np.arange(0, 17, 4)
    indices = np.tile(np.arange(4), 4)
    data = np.array(A).reshape(-1)
    b = O.spmv(indptr, indices, data, np.ones(4))
    x, it = O.solve("bicgstab2", indptr, indices, data, b, itmax=1000, eps=1e-10)
    got = "".join("%g\n" % v for v in x)
    ref = open(O.os.path.join(O.os.path.dirname(__file__), "..", "tests", "golden", "ref_test_CG.txt")).read()
    assert got == ref


FEM_NAMES = ["fem_planestrain_sample", "fem_q4_jitter", "fem_q4_heat_jitter", "fem_t3_jitter", "fem_h8_jitter",
             "fem_solid_sample"]


@pytest.mark.parametrize("name", FEM_NAMES)
def test_fem_explicit_mesh_assembly_bitexact(name):
    """The general path on explicit meshes (permuted node ids, jittered coordinates, per-element
    moduli, prescribed nonzero values, uniform body forces and edge tractions): numbering, CSR
    pattern, values and F of the oracle
    against the reference's SetDirichlet / Renumbering / Assembling / CSR(LILCSR&) run, bit for
    bit; the element matrix of element 0 too (T3, Q4, Q4 heat, H8)."""
    g = load(name)
    kind = int(g["kind"][0])
    nd = {0: 2, 1: 1, 2: 3, 3: 2}[kind]
    nn = len(g["coords"])
    fixed = np.zeros(nn * nd, np.uint8)
    uf = np.zeros(nn * nd)
    for n, d, v in g["fixed"]:
        fixed[int(n) * nd + int(d)] = 1
        uf[int(n) * nd + int(d)] = v
    n2g, N = O.renumber(nn, nd, fixed)
    V, t = g["Vt"]
    body = None if np.isnan(g["body"]).any() else tuple(g["body"])
    ip, ix, dat, F = O.assemble(kind, g["conn"], g["coords"], g["E"], n2g, N, V, t, ufixed=uf, body=body)
    L = g["loads"]
    F = O.neumann(F, L[:, 0].astype(int), L[:, 1].astype(int), L[:, 2], nd, n2g)
    if len(g["edges"]):
        F = O.edge_loads(F, g["edges"], g["coords"], g["traction"], t, n2g)
    for a, b in ((n2g, "n2g"), (ip, "indptr"), (ix, "indices"), (dat, "data"), (F, "F")):
        assert same(g[b], a), b
    X = g["coords"][g["conn"][0]]
    assert same(g["Ke0"], O.ke(kind, X, g["E"][0], V, t))
