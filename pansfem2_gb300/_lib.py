"""ctypes binding of the C ABI in include/pansfem2_gpu.h.

The shared library is built in-tree by pansfem2_gb300/build.py.  There is no
CPU fallback: if the library is missing or no CUDA device is present, every
entry point raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpansfem2_gb300.so")

PSF_OK, PSF_NOT_CONVERGED, PSF_FELL_BACK, PSF_BAD_INPUT, PSF_CUDA_ERROR, PSF_TIMEOUT, PSF_NOT_FINITE = range(7)
PSF_KERNEL_PCG_CSR, PSF_KERNEL_OPT = 0, 1
STATUS_NAMES = ["OK", "NOT_CONVERGED", "FELL_BACK", "BAD_INPUT", "CUDA_ERROR", "TIMEOUT", "NOT_FINITE"]

SOLVERS = {
    "csr_jacobi_f64": 0,
    "ebe_jacobi_f64": 1,
    "ir_jacobi_f32": 2,
    "ir_mg_f32": 3,
    "csr_cg_f64": 4,
    "csr_bicgstab_f64": 5,
    "ir_learned_f32": 6,
    "csr_scaling_bicgstab_f64": 7,
    "csr_bicgstab2_f64": 8,
    "csr_ilu0_cg_f64": 9,
    "csr_ilu0_bicgstab_f64": 10,
}

# every symbol declared in include/pansfem2_gpu.h
EXPORTS = [
    "psf_create", "psf_destroy", "psf_last_error", "psf_kernel_launches", "psf_set_launch_shape",
    "psf_get_launch_shape", "psf_diag_barrier_timeout", "psf_sizes", "psf_set_dirichlet", "psf_set_loads",
    "psf_element_matrix", "psf_build_csr", "psf_assemble", "psf_spmv", "psf_ebe_matvec", "psf_mg_precondition", "psf_solve",
    "psf_filter_setup", "psf_filter_forward", "psf_filter_backward", "psf_sensitivity_filter",
    "psf_compliance_sensitivity",
    "psf_oc_update", "psf_mma_init", "psf_mma_update", "psf_conlin_init", "psf_conlin_update",
    "psf_heaviside_forward", "psf_heaviside_backward", "psf_simp_begin", "psf_simp_step",
    "psf_simp_step_host", "psf_simp_fields", "psf_device_ptr", "psf_sync",
    "psf_csr_spmv", "psf_csr_solve", "psf_list_filter", "psf_csr_solve_noalloc", "psf_csr_solve_ilu0",
    "psf_csr_ilu0",
    "psf_fem_create", "psf_fem_destroy", "psf_fem_set_dirichlet", "psf_fem_set_loads", "psf_fem_assemble",
    "psf_fem_get_system", "psf_fem_solve", "psf_fem_reaction", "psf_fem_set_body_force", "psf_fem_set_edge_loads",
    "psf_fem_timings",
    "psf_unet_create", "psf_unet_destroy", "psf_unet_nparams", "psf_unet_set_params", "psf_unet_get_params",
    "psf_unet_forward_host", "psf_unet_loss_grad_host", "psf_unet_conv", "psf_unet_get_out_scale",
    "psf_unet_set_out_scale",
    "psf_learned_attach", "psf_learned_apply", "psf_trainset_create", "psf_trainset_destroy", "psf_trainset_size",
    "psf_learned_harvest", "psf_learned_train", "psf_learned_eval", "psf_export_vtk", "psf_export_wait",
    "psf_batch_create", "psf_batch_destroy", "psf_batch_begin", "psf_batch_step", "psf_batch_results",
    "psf_batch_profile", "psf_mma_create", "psf_mma_set_parameters", "psf_mma_update_host", "psf_mma_destroy",
    "psf_batch_fields",
]


class PsfError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else status}: {msg}")
        self.status = status


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("outer_iterations", C.c_int), ("fell_back", C.c_int),
                ("rel_residual", C.c_double), ("rel_residual_recurrence", C.c_double),
                ("seconds", C.c_double), ("kernel_seconds", C.c_double), ("kernel_launches", C.c_int),
                ("pad_", C.c_int)]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


class SimpParams(C.Structure):
    _fields_ = [("E1", C.c_double), ("E0", C.c_double), ("p", C.c_double),
                ("vf", C.c_double), ("R", C.c_double), ("scale0", C.c_double), ("scale1", C.c_double),
                ("rho0", C.c_double), ("optimizer", C.c_int),
                ("oc_iota", C.c_double), ("oc_lmin", C.c_double), ("oc_lmax", C.c_double),
                ("oc_leps", C.c_double), ("oc_move", C.c_double),
                ("mma_raa0", C.c_double), ("mma_albefa", C.c_double), ("mma_move", C.c_double),
                ("mma_asyinit", C.c_double), ("mma_asydecr", C.c_double), ("mma_asyincr", C.c_double),
                ("mma_eps", C.c_double), ("mma_a0", C.c_double), ("mma_c", C.c_double), ("mma_d", C.c_double),
                ("mma_xmin", C.c_double), ("mma_xmax", C.c_double),
                ("solver", C.c_int), ("cg_itmax", C.c_int), ("cg_eps", C.c_double), ("warm_start", C.c_int),
                ("heaviside", C.c_int), ("beta", C.c_double), ("beta_every", C.c_int), ("beta_mult", C.c_double)]


class IterInfo(C.Structure):
    _fields_ = [("f", C.c_double), ("g", C.c_double), ("lambda_", C.c_double), ("newton_steps", C.c_int),
                ("converged", C.c_int), ("solve", SolveInfo), ("phase_seconds", C.c_double * 6)]

    def asdict(self):
        d = {"f": self.f, "g": self.g, "lambda": self.lambda_, "newton_steps": self.newton_steps,
             "converged": self.converged}
        d["solve"] = self.solve.asdict()
        d["phase_seconds"] = list(self.phase_seconds)
        return d


_lib = None


def load(path=LIB_PATH):
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library not built: {path} (run pansfem2_gb300/build.py)")
    lib = C.CDLL(path)
    vp, dp, ip, i64p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.POINTER(C.c_int64)
    fp = C.POINTER(C.c_float)
    lib.psf_last_error.restype = C.c_char_p
    sig = {
        "psf_create": [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                       C.c_double, C.c_double, C.c_double],
        "psf_destroy": [vp],
        "psf_sizes": [vp, i64p, i64p, ip, i64p, i64p],
        "psf_set_dirichlet": [vp, C.c_int, ip, ip, dp, C.POINTER(C.c_int32)],
        "psf_set_loads": [vp, C.c_int, ip, ip, dp],
        "psf_element_matrix": [vp, C.c_double, dp],
        "psf_build_csr": [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
        "psf_assemble": [vp, dp, dp, dp],
        "psf_spmv": [vp, dp, dp],
        "psf_ebe_matvec": [vp, dp, dp],
        "psf_mg_precondition": [vp, dp, dp],
        "psf_solve": [vp, C.c_int, C.c_int, C.c_double, dp, C.POINTER(SolveInfo)],
        "psf_filter_setup": [vp, C.c_double],
        "psf_filter_forward": [vp, dp, dp],
        "psf_filter_backward": [vp, dp, dp],
        "psf_sensitivity_filter": [vp, C.c_int, dp, dp, dp],
        "psf_compliance_sensitivity": [vp, dp, C.c_double, C.c_double, C.c_double, C.c_double, dp, dp],
        "psf_oc_update": [vp, dp, dp, dp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                          C.c_double, C.c_double, dp],
        "psf_mma_init": [vp] + [C.c_double] * 13,
        "psf_mma_update": [vp, dp, C.c_double, dp, C.c_double, dp, ip],
        "psf_conlin_init": [vp] + [C.c_double] * 8,
        "psf_heaviside_forward": [vp, C.c_double, dp, dp],
        "psf_heaviside_backward": [vp, C.c_double, dp, dp, dp],
        "psf_conlin_update": [vp, dp, C.c_double, dp, C.c_double, dp, ip],
        "psf_simp_begin": [vp, C.POINTER(SimpParams), dp],
        "psf_simp_step": [vp, C.POINTER(IterInfo)],
        "psf_simp_step_host": [vp, dp, dp, dp, dp, C.POINTER(IterInfo)],
        "psf_simp_fields": [vp, dp, dp, dp, dp, dp],
        "psf_device_ptr": [vp, C.c_char_p, C.POINTER(C.c_void_p)],
        "psf_sync": [vp],
        "psf_csr_spmv": [C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, dp, dp],
        "psf_csr_solve": [C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, dp, C.c_int, C.c_int,
                          C.c_double, dp, C.POINTER(SolveInfo)],
        "psf_list_filter": [C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, dp, dp],
        "psf_fem_create": [C.c_int, C.c_longlong, dp, C.c_longlong, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_void_p)],
        "psf_fem_destroy": [vp],
        "psf_fem_set_dirichlet": [vp, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, ip],
        "psf_fem_set_loads": [vp, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp],
        "psf_fem_assemble": [vp, dp, C.c_double, C.c_double, C.POINTER(C.c_longlong)],
        "psf_fem_get_system": [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, dp],
        "psf_fem_solve": [vp, C.c_int, C.c_int, C.c_double, dp, C.POINTER(SolveInfo)],
        "psf_fem_reaction": [vp, dp, dp],
        "psf_fem_timings": [vp, dp, dp, dp],
        "psf_kernel_launches": [C.POINTER(C.c_longlong)],
        "psf_set_launch_shape": [vp, C.c_int, C.c_int, C.c_int, C.c_int],
        "psf_get_launch_shape": [vp, C.c_int, ip, ip, ip],
        "psf_diag_barrier_timeout": [vp, C.c_int, C.c_int64],
        "psf_fem_set_body_force": [vp, C.c_double, C.c_double],
        "psf_fem_set_edge_loads": [vp, C.c_int, C.POINTER(C.c_int32), C.c_double, C.c_double],
        # device pointers and a stream handle
        "psf_csr_solve_ilu0": [C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, dp, dp, C.c_int, C.c_int,
                               C.c_double, dp, C.POINTER(SolveInfo)],
        "psf_csr_ilu0": [C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_int32), dp, dp, dp, dp, dp],
        "psf_csr_solve_noalloc": [C.c_int, C.c_int64, vp, vp, vp, vp, vp, C.c_int, C.c_double, vp,
                                  C.POINTER(SolveInfo)],
        # learned preconditioner network
        "psf_unet_create": [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.POINTER(C.c_void_p)],
        "psf_unet_destroy": [vp],
        "psf_unet_nparams": [vp],
        "psf_unet_set_params": [vp, fp, C.c_int],
        "psf_unet_get_params": [vp, fp, C.c_int],
        "psf_unet_forward_host": [vp, C.c_int, fp, fp],
        "psf_unet_loss_grad_host": [vp, C.c_int, fp, fp, fp, dp, fp, fp],
        "psf_unet_conv": [C.c_int] * 8 + [fp, fp, fp, C.c_int, fp],
        "psf_unet_get_out_scale": [vp, fp],
        "psf_unet_set_out_scale": [vp, C.c_float],
        "psf_learned_attach": [vp, vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int],
        "psf_learned_apply": [vp, dp, dp],
        "psf_trainset_create": [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)],
        "psf_trainset_destroy": [vp],
        "psf_trainset_size": [vp],
        "psf_learned_harvest": [vp, vp, C.c_int, ip, C.c_int],
        "psf_learned_train": [vp, vp, C.c_int, C.c_int, C.c_float, C.c_uint64, C.c_int, dp],
        "psf_learned_eval": [vp, vp, C.c_int, C.c_int, C.c_int, dp],
        "psf_export_vtk": [vp, C.c_char_p, C.c_int],
        "psf_batch_create": [C.c_int, ip, ip, ip, ip, dp, C.c_int, C.c_int, C.POINTER(C.c_void_p)],
        "psf_batch_destroy": [vp],
        "psf_batch_begin": [vp, C.POINTER(SimpParams)],
        "psf_batch_step": [vp, C.c_int, dp],
        "psf_batch_results": [vp, dp],
        "psf_batch_profile": [vp, dp],
        "psf_batch_fields": [vp, C.c_int, dp, dp, dp],
        "psf_export_wait": [vp],
        "psf_mma_create": [C.c_int, C.c_int, C.c_double, dp, dp, dp, dp, dp, C.POINTER(C.c_void_p)],
        "psf_mma_set_parameters": [vp] + [C.c_double] * 7,
        "psf_mma_update_host": [vp, dp, C.c_double, dp, dp, dp, ip],
        "psf_mma_destroy": [vp],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    _lib = lib
    return lib


def check(status, allow=(PSF_OK,)):
    if status in allow:
        return status
    msg = load().psf_last_error().decode(errors="replace")
    raise PsfError(status, msg)


def ptr(a, t=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(t))


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def kernel_launches():
    """Kernel launches this thread has made through the library (psf_kernel_launches)."""
    n = C.c_longlong()
    check(load().psf_kernel_launches(C.byref(n)))
    return n.value
