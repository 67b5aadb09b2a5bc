"""Entry points on the reference's general data structures (host arrays):
CSR<T>::operator*, ScalingCG / CG on any CSR matrix, DensityFilter with
explicit neighbour lists."""
import ctypes as C

import numpy as np

from ._lib import PSF_NOT_CONVERGED, PSF_OK, SOLVERS, SolveInfo, check, f64, i32, load, ptr


def csr_spmv(indptr, indices, data, x):
    """CSR<T>::operator* (CSR.h:108-122) on the GPU."""
    L = load()
    indptr, indices, data, x = i32(indptr), i32(indices), f64(data), f64(x)
    n = len(indptr) - 1
    y = np.zeros(n)
    check(L.psf_csr_spmv(n, ptr(indptr, C.c_int32), ptr(indices, C.c_int32), ptr(data), ptr(x), ptr(y)))
    return y


def csr_solve(indptr, indices, data, b, solver="csr_jacobi_f64", itmax=100000, eps=1e-10):
    """ScalingCG (CG.h:419-453) or CG (CG.h:123-154) on the GPU; returns (x, info).
    A solve that hits itmax returns its last iterate with status NOT_CONVERGED."""
    L = load()
    indptr, indices, data, b = i32(indptr), i32(indices), f64(data), f64(b)
    n = len(indptr) - 1
    x = np.zeros(n)
    info = SolveInfo()
    st = check(L.psf_csr_solve(n, ptr(indptr, C.c_int32), ptr(indices, C.c_int32), ptr(data), ptr(b),
                               SOLVERS[solver], int(itmax), float(eps), ptr(x), C.byref(info)),
               allow=(PSF_OK, PSF_NOT_CONVERGED))
    d = info.asdict()
    d["status"] = st
    return x, d


def csr_ilu0(indptr, indices, data, m=None, b=None):
    """ILU0 (CG.h:257-284) of the matrix on its pattern (m given: used as the factor), and with
    b, PreILU0 (CG.h:288-315) of b; returns (factor values, v or None)."""
    L = load()
    indptr, indices, data = i32(indptr), i32(indices), f64(data)
    n = len(indptr) - 1
    mo = np.zeros(len(indices))
    v = None if b is None else np.zeros(n)
    check(L.psf_csr_ilu0(n, ptr(indptr, C.c_int32), ptr(indices, C.c_int32), ptr(data),
                         None if m is None else ptr(f64(m)), None if b is None else ptr(f64(b)), ptr(mo),
                         None if v is None else ptr(v)))
    return mo, v


def csr_solve_ilu0(indptr, indices, data, m, b, solver="csr_ilu0_cg_f64", itmax=100000, eps=1e-10):
    """ILU0CG / ILU0BiCGSTAB with a given factor m (None: factored here); returns (x, info)."""
    L = load()
    indptr, indices, data, b = i32(indptr), i32(indices), f64(data), f64(b)
    n = len(indptr) - 1
    x = np.zeros(n)
    info = SolveInfo()
    st = check(L.psf_csr_solve_ilu0(n, ptr(indptr, C.c_int32), ptr(indices, C.c_int32), ptr(data),
                                    None if m is None else ptr(f64(m)), ptr(b), SOLVERS[solver], int(itmax),
                                    float(eps), ptr(x), C.byref(info)), allow=(PSF_OK, PSF_NOT_CONVERGED))
    d = info.asdict()
    d["status"] = st
    return x, d


def list_filter(nb_ptr, nb_idx, w, v):
    """DensityFilter GetFilteredVariables / GetFilteredSensitivitis (DensityFilter.h:44-71)."""
    L = load()
    nb_ptr, nb_idx, w, v = i32(nb_ptr), i32(nb_idx), f64(w), f64(v)
    n = len(nb_ptr) - 1
    out = np.zeros(n)
    check(L.psf_list_filter(n, ptr(nb_ptr, C.c_int32), ptr(nb_idx, C.c_int32), ptr(w), ptr(v), ptr(out)))
    return out
