"""Failure detection on the GPU, without a GPU fault: every failure is made on the
host (a block that never arrives, a zero diagonal, non-finite inputs) and the
library must report it through its status codes, with the context usable after.

* a grid barrier whose last block never arrives: the other blocks' bounded waits
  run out, PSF_TIMEOUT comes back within the wait limit, every block returned (the
  next launch on the same context works);
* a zero diagonal entry under ScalingCG (the reference divides by it and runs on
  with inf / NaN): PSF_BAD_INPUT before any iteration, through the host-array and
  the device-array entry points;
* a non-finite right-hand side: PSF_NOT_FINITE;
* a non-finite design in the host-buffer SIMP step: PSF_NOT_FINITE, no device work.
"""
import ctypes as C
import time

import numpy as np
import pytest

from pansfem2_gb300 import problems as PB
from tests.cases import load

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import pansfem2_gb300 as P
    from pansfem2_gb300 import _lib
    P.load()
    return P, _lib, torch


def test_barrier_wait_runs_out_and_reports_timeout(gpu):
    P, lib, _ = gpu
    with P.Problem(PB.cantilever_q4(12, 6)) as prob:
        prob.setup_bc()
        for blocks in (2, 16):
            t0 = time.perf_counter()
            st = lib.load().psf_diag_barrier_timeout(prob.h, blocks, 20000)
            dt = time.perf_counter() - t0
            assert st == lib.PSF_TIMEOUT, st
            assert "exceeded its limit" in lib.load().psf_last_error().decode()
            assert dt < 2.0, dt
        # the context is usable after the timed-out launch
        prob.assemble(np.full(prob.ne, 0.5 ** 3))
        u, info = prob.solve("csr_jacobi_f64", eps=1e-10)
        assert info["status"] == lib.PSF_OK and info["rel_residual"] < 1e-9


def test_zero_diagonal_is_rejected(gpu):
    P, lib, torch = gpu
    from pansfem2_gb300 import generic
    g = load("cantilever_12x6_oc")
    ip, ix, d, F = g["indptr"], g["indices"], g["data"].copy(), g["F0"]
    row = 5
    q = ip[row] + int(np.nonzero(ix[ip[row]:ip[row + 1]] == row)[0][0])
    d[q] = 0.0
    with pytest.raises(lib.PsfError) as e:
        generic.csr_solve(ip, ix, d, F, "csr_jacobi_f64", eps=1e-10)
    assert e.value.status == lib.PSF_BAD_INPUT and "diagonal" in str(e.value)
    # plain CG does not scale by the diagonal: the intact matrix goes through it as before
    generic.csr_solve(ip, ix, g["data"], F, "csr_cg_f64", eps=1e-10)
    # the allocation-free entry point reports it the same way
    dev = torch.device("cuda", 0)
    t = [torch.as_tensor(np.asarray(a, dt), device=dev) for a, dt in
         ((ip, np.int32), (ix, np.int32), (d, np.float64), (F, np.float64))]
    x = torch.zeros_like(t[3])
    st = lib.load().psf_csr_solve_noalloc(len(F), len(ix), *(C.c_void_p(a.data_ptr()) for a in t),
                                          C.c_void_p(x.data_ptr()), 1000, 1e-10, None, None)
    torch.cuda.synchronize()
    assert st == lib.PSF_BAD_INPUT and "diagonal" in lib.load().psf_last_error().decode()


def test_non_finite_right_hand_side(gpu):
    P, lib, _ = gpu
    from pansfem2_gb300 import generic
    g = load("cantilever_12x6_oc")
    F = g["F0"].copy()
    F[3] = np.nan
    with pytest.raises(lib.PsfError) as e:
        generic.csr_solve(g["indptr"], g["indices"], g["data"], F, "csr_jacobi_f64", eps=1e-10)
    assert e.value.status == lib.PSF_NOT_FINITE


def test_non_finite_design_is_rejected(gpu):
    P, lib, _ = gpu
    pr = PB.mbb_q4(16, 8)
    with P.Problem(pr) as prob:
        prob.setup_bc()
        prob.simp_begin(solver="ir_mg_f32", cg_eps=1e-8)
        s = np.full(prob.ne, pr["vf"])
        s_next, rho = np.zeros(prob.ne), np.zeros(prob.ne)
        s[7] = np.nan
        l0 = P.kernel_launches()
        with pytest.raises(lib.PsfError) as e:
            prob.simp_step_host(s, s_next, rho)
        assert e.value.status == lib.PSF_NOT_FINITE and "design entry 7" in str(e.value)
        assert P.kernel_launches() == l0
        # a finite design goes through on the same context
        s[7] = pr["vf"]
        info = prob.simp_step_host(s, s_next, rho)
        assert info["status"] == lib.PSF_OK
