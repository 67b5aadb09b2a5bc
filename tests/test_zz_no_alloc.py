"""psf_csr_solve_noalloc: the ScalingCG solve for callers that cannot allocate
device memory when they solve (a host whose pool allocator owns the device
heap, a real-time loop that forbids allocation after start-up).  It takes
device-resident inputs and keeps its scratch in a fixed file-scope device
array, so its answer must match psf_csr_solve (which copies host arrays and
allocates) within the solver tolerance, call after call; a malformed matrix
is rejected before any kernel indexes through it; after its set-up call the
solve takes no device memory.

This file is collected last on purpose: a failure here leaves every other
test already run.  It passes alone in a fresh process and after the others.
"""
import ctypes as C
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests.cases import load

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL_U = 1e-8   # same bar as the other solver parity tests


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pansfem2_gb300 import _lib, generic
    return torch, _lib, generic


def rel(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(b)), 1e-300)


def call_noalloc(torch, lib, ip, ix, data, b, itmax=100000, eps=1e-10, nnz=None):
    dev = torch.device("cuda", 0)
    t_ip = torch.as_tensor(np.asarray(ip, np.int32), device=dev)
    t_ix = torch.as_tensor(np.asarray(ix, np.int32), device=dev)
    t_d = torch.as_tensor(np.asarray(data, np.float64), device=dev)
    t_b = torch.as_tensor(np.asarray(b, np.float64), device=dev)
    t_x = torch.full_like(t_b, float("nan"))   # whatever the caller's buffer held before
    info = lib.SolveInfo()
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()
    st = lib.load().psf_csr_solve_noalloc(len(b), len(ix) if nnz is None else nnz, C.c_void_p(t_ip.data_ptr()),
                                          C.c_void_p(t_ix.data_ptr()), C.c_void_p(t_d.data_ptr()),
                                          C.c_void_p(t_b.data_ptr()), C.c_void_p(t_x.data_ptr()), itmax, eps, stream,
                                          C.byref(info))
    torch.cuda.synchronize()
    return st, t_x.cpu().numpy(), info


@pytest.mark.parametrize("case", ["cantilever_12x6_oc", "cantilever_60x30_oc"])
def test_noalloc_matches_existing_entry_point_twice(env, case):
    torch, lib, generic = env
    g = load(case)
    ip, ix, d, F = g["indptr"], g["indices"], g["data"], g["F0"]
    rng = np.random.default_rng(9)
    rhs = [F, F * 0.5 + rng.standard_normal(len(F)) * np.abs(F).max()]
    for b in rhs:   # two calls in a row; the second reuses the scratch the first left behind
        ref, rinfo = generic.csr_solve(ip, ix, d, b, "csr_jacobi_f64", eps=1e-10)
        st, x, info = call_noalloc(torch, lib, ip, ix, d, b)
        assert st == lib.PSF_OK, lib.load().psf_last_error()
        # the same ScalingCG; the context's solve sums its rows in a different order (sliced copy)
        assert abs(info.iterations - rinfo["iterations"]) <= max(2, rinfo["iterations"] // 50)
        assert rel(x, ref) < TOL_U
        # the FP64 true residual of the result, as the other solve entry points report it
        assert 0.0 < info.rel_residual < 1e-9, info.rel_residual
        r = b - (np.add.reduceat(d * x[ix], ip[:-1]) if len(ix) else 0.0)
        assert abs(info.rel_residual - np.linalg.norm(r) / np.linalg.norm(b)) <= 1e-3 * info.rel_residual + 1e-15
    assert rel(x, ref) < TOL_U


def test_noalloc_matches_reference_solution(env):
    torch, lib, generic = env
    g = load("cantilever_12x6_oc")
    st, x, info = call_noalloc(torch, lib, g["indptr"], g["indices"], g["data"], g["F0"])
    assert st == lib.PSF_OK and rel(x, g["result0"]) < TOL_U


def test_noalloc_rejects_sizes_beyond_the_scratch(env):
    torch, lib, generic = env
    n = 262144 + 1
    dummy = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = C.c_void_p(dummy.data_ptr())
    st = lib.load().psf_csr_solve_noalloc(n, 4, p, p, p, p, p, 10, 1e-8, None, None)
    assert st == lib.PSF_BAD_INPUT
    assert "262144" in lib.load().psf_last_error().decode()


@pytest.mark.parametrize("fault", ["column_out_of_range", "negative_column", "indptr_decreasing",
                                   "indptr_end_not_nnz", "indptr_start_not_zero"])
def test_noalloc_rejects_malformed_matrix_before_solving(env, fault):
    """The malformed matrix is planted on the host; the device check reads only the flat arrays
    and the call returns PSF_BAD_INPUT after that one kernel, before the diagonal search or the
    solve index through the matrix."""
    torch, lib, generic = env
    g = load("cantilever_12x6_oc")
    ip, ix, d = g["indptr"].copy(), g["indices"].copy(), g["data"].copy()
    nnz = len(ix)
    if fault == "column_out_of_range":
        ix[len(ix) // 2] = len(ip) - 1 + 5
    elif fault == "negative_column":
        ix[3] = -1
    elif fault == "indptr_decreasing":
        ip[4], ip[5] = ip[5], ip[4]
    elif fault == "indptr_end_not_nnz":
        nnz = nnz - 1
    else:
        ip = ip + 1
    l0 = lib.kernel_launches()
    st, x, info = call_noalloc(torch, lib, ip, ix, d, g["F0"], nnz=nnz)
    assert st == lib.PSF_BAD_INPUT, st
    assert "malformed CSR" in lib.load().psf_last_error().decode()
    assert lib.kernel_launches() - l0 == 1   # the check alone ran
    # the entry point still works afterwards
    st, x, info = call_noalloc(torch, lib, g["indptr"], g["indices"], g["data"], g["F0"])
    assert st == lib.PSF_OK and rel(x, g["result0"]) < TOL_U


_MEMORY_PROBE = r"""
import ctypes as C, json, sys
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from pansfem2_gb300 import _lib as lib
from tests.cases import load
g = load("cantilever_60x30_oc")
dev = torch.device("cuda", 0)
t = [torch.as_tensor(np.asarray(a, dt), device=dev) for a, dt in
     ((g["indptr"], np.int32), (g["indices"], np.int32), (g["data"], np.float64), (g["F0"], np.float64))]
x = torch.zeros_like(t[3])
torch.cuda.synchronize()
L = lib.load()
free0 = torch.cuda.mem_get_info(0)[0]
st0 = L.psf_csr_solve_noalloc(0, 0, None, None, None, None, None, 0, 0.0, None, None)
torch.cuda.synchronize()
free1 = torch.cuda.mem_get_info(0)[0]
info = lib.SolveInfo()
sts = []
for _ in range(2):
    sts.append(L.psf_csr_solve_noalloc(len(g["F0"]), len(g["indices"]), *(C.c_void_p(a.data_ptr()) for a in t[:4]),
                                       C.c_void_p(x.data_ptr()), 100000, 1e-10, None, C.byref(info)))
torch.cuda.synchronize()
free2 = torch.cuda.mem_get_info(0)[0]
print(json.dumps({"setup_status": st0, "solve_status": sts, "free0": free0, "free1": free1, "free2": free2,
                  "res": info.rel_residual}))
"""


def test_noalloc_setup_then_solves_take_no_device_memory(env):
    """In a fresh process with lazy module loading, the set-up call (n == 0) is where the driver
    takes the scratch array and the solve kernels' code; the two solves after it take no device
    memory (cudaMemGetInfo unchanged)."""
    envv = dict(os.environ, CUDA_MODULE_LOADING="LAZY")
    p = subprocess.run([sys.executable, "-c", _MEMORY_PROBE, ROOT], capture_output=True, text=True, env=envv,
                       cwd=ROOT, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    r = json.loads(p.stdout.strip().splitlines()[-1])
    assert r["setup_status"] == 0 and r["solve_status"] == [0, 0], r
    assert r["free0"] - r["free1"] >= 0, r
    assert r["free2"] == r["free1"], r
    assert r["res"] < 1e-9, r
