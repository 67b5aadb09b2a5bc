"""psf_csr_solve_noalloc: the ScalingCG solve for callers that cannot allocate
device memory when they solve (a host whose pool allocator owns the device
heap, a real-time loop that forbids allocation after start-up).  It takes
device-resident inputs and keeps its scratch in a fixed file-scope device
array, so its answer must match psf_csr_solve (which copies host arrays and
allocates) within the solver tolerance, call after call.

This file is collected last on purpose: a failure here leaves every other
test already run.  It passes alone in a fresh process and after the others.
"""
import ctypes as C

import numpy as np
import pytest

from tests.cases import load

pytestmark = pytest.mark.gpu

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


def call_noalloc(torch, lib, ip, ix, data, b, itmax=100000, eps=1e-10):
    dev = torch.device("cuda", 0)
    t_ip = torch.as_tensor(np.asarray(ip, np.int32), device=dev)
    t_ix = torch.as_tensor(np.asarray(ix, np.int32), device=dev)
    t_d = torch.as_tensor(np.asarray(data, np.float64), device=dev)
    t_b = torch.as_tensor(np.asarray(b, np.float64), device=dev)
    t_x = torch.full_like(t_b, float("nan"))   # whatever the caller's buffer held before
    info = lib.SolveInfo()
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    st = lib.load().psf_csr_solve_noalloc(len(b), C.c_void_p(t_ip.data_ptr()), C.c_void_p(t_ix.data_ptr()),
                                          C.c_void_p(t_d.data_ptr()), C.c_void_p(t_b.data_ptr()),
                                          C.c_void_p(t_x.data_ptr()), itmax, eps, stream, C.byref(info))
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
        assert info.iterations == rinfo["iterations"]
        assert rel(x, ref) < TOL_U
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
    st = lib.load().psf_csr_solve_noalloc(n, p, p, p, p, p, 10, 1e-8, None, None)
    assert st == lib.PSF_BAD_INPUT
    assert "262144" in lib.load().psf_last_error().decode()
