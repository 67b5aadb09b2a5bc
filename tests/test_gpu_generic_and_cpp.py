"""GPU checks of the entry points on general data structures and of the C++
mirror of the reference API (a sample loop compiled against it)."""
import os
import subprocess

import numpy as np
import pytest

from oracle import pyoracle as O
from pansfem2_gb300 import problems as PB
from tests.cases import CASES, load

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pansfem2_gb300 import generic
    return generic


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300)


def test_csr_spmv_and_solvers_on_reference_csr(gpu):
    """The reference's own CSR (12x6 cantilever) through psf_csr_*: SpMV,
    ScalingCG and CG against the reference's results (golden)."""
    g = load("cantilever_12x6_oc")
    ip, ix, d, F = g["indptr"], g["indices"], g["data"], g["F0"]
    x = np.random.default_rng(2).standard_normal(len(F))
    assert rel(gpu.csr_spmv(ip, ix, d, x), O.spmv(ip, ix, d, x)) < 1e-12
    u, info = gpu.csr_solve(ip, ix, d, F, "csr_jacobi_f64", eps=1e-10)
    assert info["status"] == 0 and rel(u, g["result0"]) < 1e-8
    u, info = gpu.csr_solve(ip, ix, d, F, "csr_cg_f64", eps=1e-10)
    assert info["status"] == 0 and rel(u, g["sol_cg"]) < 1e-8


def test_csr_solve_not_converged_returns_last_iterate(gpu):
    g = load("cantilever_12x6_oc")
    ip, ix, d, F = g["indptr"], g["indices"], g["data"], g["F0"]
    u, info = gpu.csr_solve(ip, ix, d, F, "csr_jacobi_f64", itmax=3, eps=1e-14)
    assert info["status"] == 1 and info["iterations"] == 3 and np.all(np.isfinite(u))


def test_list_filter_on_reference_lists(gpu):
    g = load("mbb_16x8_mma")
    s = np.random.default_rng(4).uniform(0, 1, len(g["nb_ptr"]) - 1)
    assert rel(gpu.list_filter(g["nb_ptr"], g["nb_idx"], g["nb_w"], s),
               O.density_filter(g["nb_ptr"], g["nb_idx"], g["nb_w"], s)) < 1e-14


def test_cpp_sample_through_the_mirrored_api(gpu, tmp_path):
    """tests/cpp/sample_mbb_gpu.cpp: the MMA sample loop against
    include/pansfem2_gb300.hpp; objective per iteration vs the oracle."""
    from pansfem2_gb300 import _lib
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "sample_mbb_gpu")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "sample_mbb_gpu.cpp"), "-o", exe,
                    "-L", libdir, "-lpansfem2_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    out = subprocess.run([exe, "48", "24", "5"], check=True, capture_output=True, text=True).stdout
    fs = [float(l.split()[3]) for l in out.splitlines() if l.startswith("k ")]
    ref = O.simp_run(CASES["mbb_48x24_mma"](), 5)
    assert len(fs) == 5
    for k in range(5):
        assert abs(fs[k] - ref["f"][k]) <= 1e-6 * abs(ref["f"][k]), (k, fs[k], ref["f"][k])
    cs = float([l for l in out.splitlines() if l.startswith("checksum")][0].split()[1])
    assert abs(cs - ref["s_final"].sum()) <= 1e-6 * len(ref["s_final"])
