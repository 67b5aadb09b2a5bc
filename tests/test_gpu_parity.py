"""GPU parity: the CUDA path through the C ABI against the oracle and the
reference's golden fixtures.

Bars: integer work (numbering, CSR pattern) and the element matrix bit-exact;
floating point within the stated tolerance of each check (the GPU sums in a
different order and scales one shared element matrix by E_e).
"""
import numpy as np
import pytest

from oracle import pyoracle as O
from pansfem2_gb300 import problems as PB
from tests.cases import CASES, load

pytestmark = pytest.mark.gpu

# tolerances (relative unless stated)
TOL_VALUES = 1e-13      # assembled CSR values: E*Ke0 vs Ke(E) per element, sums in the same order
TOL_OPERATOR = 1e-12    # K.x, CSR and matrix-free
TOL_FILTER = 1e-14
TOL_SENS = 1e-9         # sensitivities/compliance from a solved u (solution error dominates)
TOL_U = 1e-8            # displacements vs the oracle's ScalingCG solution
TOL_RHO = 1e-6          # densities, max-abs over the first 10 SIMP iterations
TOL_F = 1e-6            # compliance, relative


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    P.load()
    return P


def geometry(pr):
    if pr["kind"] == PB.H8_SOLID:
        return (O.h8_nodes(pr["lx"], pr["ly"], pr["lz"], pr["nx"], pr["ny"], pr["nz"]),
                O.h8_elements(pr["nx"], pr["ny"], pr["nz"]), 3)
    return O.q4_nodes(pr["lx"], pr["ly"], pr["nx"], pr["ny"]), O.q4_elements(pr["nx"], pr["ny"]), 2


def rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


CSR_CASES = [n for n in sorted(CASES) if "indptr" in load(n)]   # fixtures that keep the reference's CSR


@pytest.mark.parametrize("name", CSR_CASES)
def test_numbering_pattern_bitexact(gpu, name):
    g, pr = load(name), CASES[name]()
    with gpu.Problem(pr) as P:
        n2g = P.setup_bc()
        assert np.array_equal(n2g, g["n2g"])
        indptr, indices = P.build_csr()
        assert np.array_equal(indptr, g["indptr"]) and np.array_equal(indices, g["indices"])


@pytest.mark.parametrize("name", CSR_CASES)
def test_element_matrix_bitexact(gpu, name):
    g, pr = load(name), CASES[name]()
    with gpu.Problem(pr) as P:
        assert np.array_equal(P.element_matrix(1.0).reshape(-1), g["Ke0"])


@pytest.mark.parametrize("name", CSR_CASES)
def test_assembly_values_and_rhs(gpu, name):
    g, pr = load(name), CASES[name]()
    coords, conn, dim = geometry(pr)
    ne, nn, nd = PB.counts(pr)
    rho0 = O.density_filter(*O.neighbors(O.centroids(conn, coords, dim), pr["R"]), np.full(ne, pr["rho0"]))
    E = pr["E1"] * np.power(rho0, pr["p"]) + pr["E0"] * (1.0 - np.power(rho0, pr["p"]))
    with gpu.Problem(pr) as P:
        P.setup_bc()
        data, F = P.assemble(E)
        assert rel(data, g["data"]) < TOL_VALUES
        assert np.array_equal(F, g["F0"])


@pytest.mark.parametrize("name", ["cantilever_12x6_oc", "heatsink_10x10_oc", "cantilever_h8_6x3x3_oc"])
def test_operator_csr_and_matrix_free(gpu, name):
    g, pr = load(name), CASES[name]()
    ne, nn, nd = PB.counts(pr)
    rng = np.random.default_rng(7)
    E = rng.uniform(1e-3, 1.0, ne)
    coords, conn, dim = geometry(pr)
    n2g, N = O.renumber(nn, nd, PB.fixed_mask(pr))
    ip, ix, dat, _ = O.assemble(pr["kind"], conn, coords, E, n2g, N, pr["V"], pr["t"])
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.assemble(E)
        for _ in range(3):
            x = rng.standard_normal(N)
            y_ref = O.spmv(ip, ix, dat, x)
            assert rel(P.spmv(x), y_ref) < TOL_OPERATOR
            assert rel(P.ebe_matvec(x), y_ref) < TOL_OPERATOR


@pytest.mark.parametrize("solver", ["csr_jacobi_f64", "ebe_jacobi_f64", "ir_jacobi_f32", "ir_mg_f32"])
@pytest.mark.parametrize("name", ["cantilever_12x6_oc", "mbb_16x8_mma", "heatsink_10x10_oc",
                                  "cantilever_h8_6x3x3_oc", "cantilever_60x30_oc"])
def test_solve_matches_oracle(gpu, name, solver):
    g, pr = load(name), CASES[name]()
    coords, conn, dim = geometry(pr)
    ne, nn, nd = PB.counts(pr)
    rho0 = O.density_filter(*O.neighbors(O.centroids(conn, coords, dim), pr["R"]), np.full(ne, pr["rho0"]))
    E = pr["E1"] * np.power(rho0, pr["p"]) + pr["E0"] * (1.0 - np.power(rho0, pr["p"]))
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.assemble(E)
        u, info = P.solve(solver, eps=1e-10)
        assert info["status"] == 0, info
        assert info["rel_residual"] < 1e-9
        assert rel(u, g["result0"]) < TOL_U


@pytest.mark.parametrize("shape", [(1, 1024, 1), (1, 256, 4), (4, 1024, 1), (8, 512, 2), (16, 256, 4)])
@pytest.mark.parametrize("name", ["cantilever_12x6_oc", "cantilever_h8_6x3x3_oc", "cantilever_60x30_oc"])
def test_fp64_pcg_launch_shapes_match_oracle(gpu, name, shape):
    """Every launch shape of the FP64 CSR PCG: one lane per row on the sliced copy (row
    counts that are not multiples of 32, 3D rows of 81 entries) and 4 / 8 / 16 lanes per row on
    the CSR itself."""
    from pansfem2_gb300 import _lib
    g, pr = load(name), CASES[name]()
    coords, conn, dim = geometry(pr)
    ne = PB.counts(pr)[0]
    rho0 = O.density_filter(*O.neighbors(O.centroids(conn, coords, dim), pr["R"]), np.full(ne, pr["rho0"]))
    E = pr["E1"] * np.power(rho0, pr["p"]) + pr["E0"] * (1.0 - np.power(rho0, pr["p"]))
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.assemble(E)
        P.set_launch_shape(_lib.PSF_KERNEL_PCG_CSR, *shape)
        assert P.launch_shape(_lib.PSF_KERNEL_PCG_CSR) == shape
        u, info = P.solve("csr_jacobi_f64", eps=1e-10)
        assert info["status"] == 0, info
        assert info["rel_residual"] < 1e-9
        assert rel(u, g["result0"]) < TOL_U


@pytest.mark.parametrize("name", ["cantilever_12x6_oc", "mbb_16x8_mma", "cantilever_h8_6x3x3_oc"])
def test_filter_forward_backward(gpu, name):
    g, pr = load(name), CASES[name]()
    ne = PB.counts(pr)[0]
    rng = np.random.default_rng(3)
    s, d = rng.uniform(0, 1, ne), rng.standard_normal(ne)
    with gpu.Problem(pr) as P:
        P.filter_setup()
        assert rel(P.filter_forward(s), O.density_filter(g["nb_ptr"], g["nb_idx"], g["nb_w"], s)) < TOL_FILTER
        assert rel(P.filter_backward(d), O.density_filter_sens(g["nb_ptr"], g["nb_idx"], g["nb_w"], d)) < TOL_FILTER


@pytest.mark.parametrize("name", ["cantilever_12x6_oc", "heatsink_10x10_oc", "cantilever_h8_6x3x3_oc"])
def test_compliance_sensitivity(gpu, name):
    g, pr = load(name), CASES[name]()
    coords, conn, dim = geometry(pr)
    rho = g["rho"][: PB.counts(pr)[0]]
    u = g["u"][: PB.counts(pr)[1] * PB.counts(pr)[2]]
    f_ref = g["f"][0]
    with gpu.Problem(pr) as P:
        P.setup_bc()
        E = pr["E1"] * np.power(rho, pr["p"]) + pr["E0"] * (1.0 - np.power(rho, pr["p"]))
        P.assemble(E)
        P.solve("csr_jacobi_f64", eps=1e-10)
        f, d = P.compliance_sensitivity(rho)
        assert abs(f - f_ref) / abs(f_ref) < TOL_SENS
        assert rel(d, g["dfdrho"][: len(d)]) < TOL_SENS


def test_oc_update_matches_oracle(gpu):
    g, pr = load("cantilever_60x30_oc"), CASES["cantilever_60x30_oc"]()
    ne = PB.counts(pr)[0]
    rng = np.random.default_rng(11)
    x = rng.uniform(0.2, 0.8, ne)
    dfdx = -rng.uniform(0.1, 3.0, ne)
    dgdx = np.full(ne, 1.0 / (pr["vf"] * ne))
    x_ref, lam_ref = O.oc_update(x, dfdx, dgdx, g["nb_ptr"], g["nb_idx"], g["nb_w"], pr["vf"], move=pr["oc_move"])
    with gpu.Problem(pr) as P:
        P.filter_setup()
        x_gpu, lam = P.oc_update(x, dfdx, dgdx)
    assert abs(lam - lam_ref) <= 1e-12 * lam_ref
    assert np.max(np.abs(x_gpu - x_ref)) < 1e-12


@pytest.mark.parametrize("arith", ["double_word", "fp64"])
def test_mma_update_matches_oracle(gpu, arith, monkeypatch):
    """Both interior-point kernels: the double-word one (default) and the FP64 one
    (PSF_OPT_F64=1, also the fallback when data leave the FP32 pair range)."""
    if arith == "fp64":
        monkeypatch.setenv("PSF_OPT_F64", "1")
    pr = CASES["mbb_48x24_mma"]()
    ne = PB.counts(pr)[0]
    rng = np.random.default_rng(5)
    mma = O.MMA(ne, 1, pr["mma_a0"], [0.0], [pr["mma_c"]], [pr["mma_d"]], np.full(ne, pr["mma_xmin"]),
                np.full(ne, pr["mma_xmax"]))
    mma.set_parameters(pr["mma_raa0"], pr["mma_albefa"], pr["mma_move"], pr["mma_asyinit"], pr["mma_asydecr"],
                       pr["mma_asyincr"], pr["mma_eps"])
    x_ref = np.full(ne, pr["vf"])
    with gpu.Problem(pr) as P:
        P.mma_init()
        x_gpu = x_ref.copy()
        for k in range(4):   # four outer steps exercise both asymptote branches
            dfdx = -rng.uniform(0.1, 2.0, ne)
            dgdx = np.full(ne, 1.0 / (pr["vf"] * ne))
            g = float(np.sum(x_ref) / (pr["vf"] * ne) - 1.0)
            x_ref, n_ref = mma.update(x_ref, 10.0, dfdx, [g], dgdx)
            x_gpu, n_gpu = P.mma_update(x_gpu, 10.0, dfdx, g, dgdx)
            assert np.max(np.abs(x_gpu - x_ref)) < 1e-7, k
            x_gpu = x_ref.copy()   # re-sync the next step's input


@pytest.mark.parametrize("solver", ["csr_jacobi_f64", "ebe_jacobi_f64", "ir_jacobi_f32", "ir_mg_f32"])
@pytest.mark.parametrize("name", ["cantilever_60x30_oc", "mbb_48x24_mma", "heatsink_10x10_oc",
                                  "cantilever_h8_6x3x3_oc"])
def test_simp_trajectory_first_iterations(gpu, name, solver):
    """Densities within 1e-6 max-abs and compliance within 1e-6 relative of the
    reference over the first iterations of the SIMP loop."""
    g, pr = load(name), CASES[name]()
    iters = int(g["iters"][0])
    ne = PB.counts(pr)[0]
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver=solver, cg_eps=1e-10)
        for k in range(iters):
            info = P.simp_step()
            fl = P.fields()
            assert abs(info["f"] - g["f"][k]) <= TOL_F * abs(g["f"][k]), (k, info["f"], g["f"][k])
            assert np.max(np.abs(fl["rho"] - g["rho"].reshape(iters, ne)[k])) < TOL_RHO, k
            assert np.max(np.abs(fl["s"] - g["s_after"].reshape(iters, ne)[k])) < TOL_RHO, k


def test_full_size_properties_mbb_1024x512(gpu):
    """At the benchmark size (1,051,650 dofs): K symmetric (x.Ky == y.Kx),
    CSR == matrix-free, and each solver reaches the FP64 true residual 1e-8."""
    pr = PB.mbb_q4(1024, 512)
    ne, nn, nd = PB.counts(pr)
    rng = np.random.default_rng(1)
    E = 1e-9 + (1 - 1e-9) * rng.uniform(0.0, 1.0, ne) ** 3
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.assemble(E)
        x, y = rng.standard_normal(P.nfree), rng.standard_normal(P.nfree)
        Kx, Ky = P.spmv(x), P.spmv(y)
        assert abs(x @ Ky - y @ Kx) <= 1e-12 * abs(x @ Ky)
        assert rel(P.ebe_matvec(x), Kx) < TOL_OPERATOR
        E = np.full(ne, 0.4 ** 3)
        P.assemble(E)
        sols = {}
        for solver in ("ebe_jacobi_f64", "ir_jacobi_f32", "ir_mg_f32"):
            u, info = P.solve(solver, itmax=200000, eps=1e-8)
            assert info["status"] == 0 and info["rel_residual"] < 1.5e-8, (solver, info)
            sols[solver] = u
        # same solution from every path (to the accuracy a 1e-8 residual buys)
        for solver in ("ir_jacobi_f32", "ir_mg_f32"):
            assert rel(sols[solver], sols["ebe_jacobi_f64"]) < 1e-5, solver


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name", ["cantilever_60x30_oc", "cantilever_h8_6x3x3_oc"])
def test_sensitivity_filters_match_oracle(gpu, name, mode):
    """SensitivityFilter (Sigmund, mode 0) and SensitivityFilter2 (Borrvall, mode 1) on the
    grid's filter against the oracle's list form (neighbour lists of the reference samples)."""
    g, pr = load(name), CASES[name]()
    coords, conn, dim = geometry(pr)
    ne = PB.counts(pr)[0]
    ptr, idx, w = O.neighbors(O.centroids(conn, coords, dim), pr["R"])
    rng = np.random.default_rng(mode + ne)
    s = rng.uniform(0.05, 1.0, ne)
    d = -rng.uniform(0.0, 10.0, ne)
    ref = O.sensitivity_filter(ptr, idx, w, s, d, mode)
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.filter_setup()
        out = P.sensitivity_filter(s, d, mode)
    assert np.max(np.abs(out - ref)) <= TOL_FILTER * np.max(np.abs(ref))


@pytest.mark.parametrize("nx,ny", [(60, 30), (61, 30), (1000, 500)])
def test_multigrid_on_grids_not_divisible_by_two(gpu, nx, ny):
    """The multigrid FCG on grids whose axes turn odd while coarsening (60x30 -> 30x15 -> 15x8
    -> ..., 61x30 from the start, 1000x500 -> ... -> 125x63 -> ...): every solve reaches the FP64
    true residual, the compliance equals the FP64 Jacobi PCG's, and the per-solve set-up (the
    Galerkin levels and the dense coarsest inverse, rebuilt every SIMP iteration) is short."""
    pr = PB.cantilever_q4(nx, ny) if nx < 100 else PB.mbb_q4(nx, ny)
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver="ir_mg_f32", cg_eps=1e-10, warm_start=True)
        infos = [P.simp_step() for _ in range(3)]
        s = P.fields()["s"]
    for i in infos:
        assert i["status"] == 0 and i["solve"]["rel_residual"] < 1e-10, i["solve"]
        assert i["solve"]["iterations"] < 200, i["solve"]
    # set-up time of a later iteration: the solve's device time outside the Krylov kernel
    # (hierarchy, coarsest inverse, true-residual check)
    setup = infos[-1]["solve"]["seconds"] - infos[-1]["solve"]["kernel_seconds"]
    assert setup < (1e-3 if nx < 100 else 5e-3), setup
    # the same design solved by the FP64 Jacobi PCG path: the same compliance
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver="ir_mg_f32", cg_eps=1e-10, warm_start=False, s0=s)
        f_mg = P.simp_step()["f"]
    with gpu.Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver="csr_jacobi_f64", cg_eps=1e-10, warm_start=False, s0=s)
        f_pcg = P.simp_step()["f"]
    assert abs(f_mg - f_pcg) <= 1e-8 * abs(f_pcg), (f_mg, f_pcg)
