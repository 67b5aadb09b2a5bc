"""The remaining Krylov solvers of CG.h on the GPU against the reference's own outputs
(tests/golden/cantilever_12x6_oc.npz, written by the reference's CG.h on the first system
of the 12x6 cantilever): ILU0 (factor values) and PreILU0 bit for bit, ScalingBiCGSTAB,
BiCGSTAB2, ILU0CG and ILU0BiCGSTAB solutions within 1e-8; the same solvers against the
oracle on a larger system (60x30 cantilever, 3,720 unknowns), and the C++ mirror's
functions of the same names."""
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as O
from tests.cases import load

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL_U = 1e-8


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pansfem2_gb300 import generic
    return generic


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300)


def test_ilu0_factor_and_apply_bitexact(gpu):
    g = load("cantilever_12x6_oc")
    m, v = gpu.csr_ilu0(g["indptr"], g["indices"], g["data"], b=g["F0"])
    assert np.array_equal(g["ilu_indptr"], g["indptr"]) and np.array_equal(g["ilu_indices"], g["indices"])
    assert np.array_equal(m, g["ilu_data"])
    assert np.array_equal(v, g["ilu_apply_F"])
    # the apply with a given factor (PreILU0(M, b))
    _, v2 = gpu.csr_ilu0(g["indptr"], g["indices"], g["data"], m=g["ilu_data"], b=g["F0"])
    assert np.array_equal(v2, g["ilu_apply_F"])


@pytest.mark.parametrize("solver,key", [("csr_scaling_bicgstab_f64", "sol_scalingbicgstab"),
                                        ("csr_bicgstab2_f64", "sol_bicgstab2"),
                                        ("csr_ilu0_cg_f64", "sol_ilu0cg"),
                                        ("csr_ilu0_bicgstab_f64", "sol_ilu0bicgstab")])
def test_solvers_match_reference_solutions(gpu, solver, key):
    g = load("cantilever_12x6_oc")
    x, info = gpu.csr_solve(g["indptr"], g["indices"], g["data"], g["F0"], solver, eps=1e-10)
    assert info["status"] == 0, info
    assert rel(x, g[key]) < TOL_U, (solver, rel(x, g[key]))


@pytest.mark.parametrize("solver,kind", [("csr_scaling_bicgstab_f64", "scaling_bicgstab"),
                                         ("csr_bicgstab2_f64", "bicgstab2"), ("csr_ilu0_cg_f64", "ilu0_cg"),
                                         ("csr_ilu0_bicgstab_f64", "ilu0_bicgstab")])
def test_solvers_match_oracle_60x30(gpu, solver, kind):
    g = load("cantilever_60x30_oc")
    x, info = gpu.csr_solve(g["indptr"], g["indices"], g["data"], g["F0"], solver, eps=1e-10)
    xo, it = O.solve(kind, g["indptr"], g["indices"], g["data"], g["F0"], eps=1e-10)
    assert info["status"] == 0 and it > 0, (info, it)
    assert rel(x, xo) < TOL_U and rel(x, g["result0"]) < TOL_U
    # the same number of iterations to rounding of the stopping test
    assert abs(info["iterations"] - it) <= max(2, it // 50), (info["iterations"], it)


def test_ilu0_factor_matches_oracle_60x30(gpu):
    g = load("cantilever_60x30_oc")
    m, v = gpu.csr_ilu0(g["indptr"], g["indices"], g["data"], b=g["F0"])
    mi, mj, md = O.ilu0(g["indptr"], g["indices"], g["data"])
    assert np.array_equal(m, md)
    x, info = gpu.csr_solve_ilu0(g["indptr"], g["indices"], g["data"], md, g["F0"], "csr_ilu0_cg_f64", eps=1e-10)
    assert info["status"] == 0 and rel(x, g["result0"]) < TOL_U


def test_cpp_mirror_solvers(gpu, tmp_path):
    """The mirror's BiCGSTAB, ScalingBiCGSTAB, BiCGSTAB2, ILU0 / ILU0CG / ILU0BiCGSTAB on the reference's
    12x6 system read from a text file; every solution within 1e-8 of the reference's."""
    from pansfem2_gb300 import _lib
    g = load("cantilever_12x6_oc")
    sysf = tmp_path / "sys.txt"
    with open(sysf, "w") as fh:
        fh.write(f"{len(g['F0'])} {len(g['indices'])}\n")
        fh.write(" ".join(map(str, g["indptr"])) + "\n" + " ".join(map(str, g["indices"])) + "\n")
        fh.write(" ".join(repr(float(v)) for v in g["data"]) + "\n" + " ".join(repr(float(v)) for v in g["F0"]) + "\n")
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "krylov_gpu")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "krylov_gpu.cpp"), "-o", exe,
                    "-L", libdir, "-lpansfem2_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([exe, str(sysf)], check=True, capture_output=True, text=True).stdout
    sols = {l.split()[0]: np.array(l.split()[1:], float) for l in out.splitlines() if l.strip()}
    for name, key in (("BiCGSTAB", "sol_bicgstab"), ("ScalingBiCGSTAB", "sol_scalingbicgstab"),
                      ("BiCGSTAB2", "sol_bicgstab2"), ("ILU0CG", "sol_ilu0cg"), ("ILU0BiCGSTAB", "sol_ilu0bicgstab")):
        assert rel(sols[name], g[key]) < TOL_U, name
