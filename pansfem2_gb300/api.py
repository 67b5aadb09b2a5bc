"""Python host over the C ABI: one Problem owns one device context.

Mirrors the reference call sequence of the SIMP samples
(sample/optimize/sample_optimize_density_{oc,mma,CONLIN}.cpp): boundary conditions
and numbering, element matrix, CSR pattern + assembly, solve, compliance and
sensitivities, density filter, OC / MMA update, or the whole iteration on the
device (simp_begin / simp_step).
"""
import ctypes as C

import numpy as np

from . import problems as PB
from ._lib import (PSF_FELL_BACK, PSF_NOT_CONVERGED, PSF_OK, SOLVERS, IterInfo, SimpParams, SolveInfo, check,
                   f64, i32, load, ptr)


class Problem:
    def __init__(self, pr):
        self.pr = dict(pr)
        self.L = load()
        h = C.c_void_p()
        kind, nx, ny, nz = pr["kind"], pr["nx"], pr["ny"], pr.get("nz", 0)
        check(self.L.psf_create(C.byref(h), kind, nx, ny, nz, float(pr.get("lx", nx)), float(pr.get("ly", ny)),
                                float(pr.get("lz", nz) or 1.0), float(pr.get("V", 0.3)), float(pr.get("t", 1.0))))
        self.h = h
        self.ne, self.nnodes, self.ndof = PB.counts(pr)
        self.nfree = None
        self.nnz = None

    def close(self):
        if getattr(self, "h", None):
            self.L.psf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---------------------------------------------------------------- launch shapes
    def set_launch_shape(self, kernel, a=0, b=256, c=2):
        """psf_set_launch_shape: kernel PSF_KERNEL_PCG_CSR (a lanes per row, b threads, c blocks
        per SM) or PSF_KERNEL_OPT (c blocks per SM)."""
        check(self.L.psf_set_launch_shape(self.h, int(kernel), int(a), int(b), int(c)))

    def launch_shape(self, kernel):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(self.L.psf_get_launch_shape(self.h, int(kernel), C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    # ---------------------------------------------------------------- set-up
    def _sizes(self):
        ne, nn, nf, nz = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        nd = C.c_int()
        check(self.L.psf_sizes(self.h, C.byref(ne), C.byref(nn), C.byref(nd), C.byref(nf), C.byref(nz)))
        self.nfree, self.nnz = nf.value, nz.value

    def set_dirichlet(self, nodes=None, dofs=None, values=None):
        nodes = i32(self.pr["fix_node"] if nodes is None else nodes)
        dofs = i32(self.pr["fix_dof"] if dofs is None else dofs)
        vals = None if values is None else f64(values)
        n2g = np.zeros(self.nnodes * self.ndof, np.int32)
        check(self.L.psf_set_dirichlet(self.h, len(nodes), ptr(nodes, C.c_int), ptr(dofs, C.c_int), ptr(vals),
                                       ptr(n2g, C.c_int32)))
        self._sizes()
        return n2g

    def set_loads(self, nodes=None, dofs=None, values=None):
        nodes = i32(self.pr["load_node"] if nodes is None else nodes)
        dofs = i32(self.pr["load_dof"] if dofs is None else dofs)
        vals = f64(self.pr["load_val"] if values is None else values)
        check(self.L.psf_set_loads(self.h, len(nodes), ptr(nodes, C.c_int), ptr(dofs, C.c_int), ptr(vals)))

    def setup_bc(self):
        n2g = self.set_dirichlet()
        self.set_loads()
        return n2g

    def element_matrix(self, E=1.0):
        nk = (8 if self.pr["kind"] == PB.H8_SOLID else 4) * self.ndof
        Ke = np.zeros(nk * nk)
        check(self.L.psf_element_matrix(self.h, float(E), ptr(Ke)))
        return Ke.reshape(nk, nk)

    def build_csr(self):
        check(self.L.psf_build_csr(self.h, None, None))
        self._sizes()
        indptr = np.zeros(self.nfree + 1, np.int32)
        indices = np.zeros(max(self.nnz, 1), np.int32)
        check(self.L.psf_build_csr(self.h, ptr(indptr, C.c_int32), ptr(indices, C.c_int32)))
        return indptr, indices[: self.nnz]

    def assemble(self, E_e):
        E_e = f64(E_e)
        if not self.nnz:
            # the pattern fixes the size of the value array the library writes
            check(self.L.psf_build_csr(self.h, None, None))
            self._sizes()
        data = np.zeros(max(self.nnz, 1))
        F = np.zeros(self.nfree)
        check(self.L.psf_assemble(self.h, ptr(E_e), ptr(data), ptr(F)))
        return data[: self.nnz], F

    def spmv(self, x):
        x = f64(x)
        y = np.zeros(self.nfree)
        check(self.L.psf_spmv(self.h, ptr(x), ptr(y)))
        return y

    def ebe_matvec(self, x):
        x = f64(x)
        y = np.zeros(self.nfree)
        check(self.L.psf_ebe_matvec(self.h, ptr(x), ptr(y)))
        return y

    def mg_precondition(self, r):
        """z = one multigrid V-cycle applied to r (psf_mg_precondition), reduced vectors."""
        r = f64(r)
        z = np.zeros(self.nfree)
        check(self.L.psf_mg_precondition(self.h, ptr(r), ptr(z)))
        return z

    def solve(self, solver="csr_jacobi_f64", itmax=100000, eps=1e-10):
        u = np.zeros(self.nfree)
        info = SolveInfo()
        st = check(self.L.psf_solve(self.h, SOLVERS[solver], int(itmax), float(eps), ptr(u), C.byref(info)),
                   allow=(PSF_OK, PSF_NOT_CONVERGED, PSF_FELL_BACK))
        d = info.asdict()
        d["status"] = st
        return u, d

    # ---------------------------------------------------------------- SIMP pieces
    def filter_setup(self, R=None):
        check(self.L.psf_filter_setup(self.h, float(self.pr["R"] if R is None else R)))

    def filter_forward(self, s):
        s = f64(s)
        out = np.zeros(self.ne)
        check(self.L.psf_filter_forward(self.h, ptr(s), ptr(out)))
        return out

    def filter_backward(self, d):
        d = f64(d)
        out = np.zeros(self.ne)
        check(self.L.psf_filter_backward(self.h, ptr(d), ptr(out)))
        return out

    def heaviside_forward(self, beta, s):
        """HeavisideFilter::GetFilteredVariables at projection sharpness beta."""
        out = np.zeros(self.ne)
        check(self.L.psf_heaviside_forward(self.h, float(beta), ptr(f64(s)), ptr(out)))
        return out

    def heaviside_backward(self, beta, s, d):
        """HeavisideFilter::GetFilteredSensitivitis of d at design s."""
        out = np.zeros(self.ne)
        check(self.L.psf_heaviside_backward(self.h, float(beta), ptr(f64(s)), ptr(f64(d)), ptr(out)))
        return out

    def sensitivity_filter(self, s, d, mode=0):
        """SensitivityFilter (mode 0) / SensitivityFilter2 (mode 1) of d at design s."""
        out = np.zeros(self.ne)
        check(self.L.psf_sensitivity_filter(self.h, int(mode), ptr(f64(s)), ptr(f64(d)), ptr(out)))
        return out

    def compliance_sensitivity(self, rho):
        rho = f64(rho)
        f = C.c_double()
        d = np.zeros(self.ne)
        pr = self.pr
        check(self.L.psf_compliance_sensitivity(self.h, ptr(rho), pr["E1"], pr["E0"], pr["p"], pr["scale0"],
                                                C.byref(f), ptr(d)))
        return f.value, d

    def oc_update(self, x, dfdx, dgdx):
        x = f64(x).copy()
        lam = C.c_double()
        pr = self.pr
        check(self.L.psf_oc_update(self.h, ptr(x), ptr(f64(dfdx)), ptr(f64(dgdx)), pr["oc_iota"], pr["oc_lmin"],
                                   pr["oc_lmax"], pr["oc_leps"], pr["oc_move"], pr["vf"], pr["scale1"],
                                   C.byref(lam)))
        return x, lam.value

    def mma_init(self):
        pr = self.pr
        check(self.L.psf_mma_init(self.h, pr["mma_a0"], 0.0, pr["mma_c"], pr["mma_d"], pr["mma_xmin"],
                                  pr["mma_xmax"], pr["mma_raa0"], pr["mma_albefa"], pr["mma_move"],
                                  pr["mma_asyinit"], pr["mma_asydecr"], pr["mma_asyincr"], pr["mma_eps"]))

    def mma_update(self, x, f, dfdx, g, dgdx):
        x = f64(x).copy()
        nt = C.c_int()
        check(self.L.psf_mma_update(self.h, ptr(x), float(f), ptr(f64(dfdx)), float(g), ptr(f64(dgdx)),
                                    C.byref(nt)), allow=(PSF_OK, PSF_NOT_CONVERGED))
        return x, nt.value

    def conlin_init(self, move=None, eps=None):
        """CONLIN(n, 1, a0, {0}, {c}, {d}, xmin, xmax) + SetParameters(move, eps) (CONLIN.h:55-74)
        from the problem's mma_a0/c/d/xmin/xmax and mma_move/mma_eps."""
        pr = self.pr
        check(self.L.psf_conlin_init(self.h, pr["mma_a0"], 0.0, pr["mma_c"], pr["mma_d"], pr["mma_xmin"],
                                     pr["mma_xmax"], pr["mma_move"] if move is None else move,
                                     pr["mma_eps"] if eps is None else eps))

    def conlin_update(self, x, f, dfdx, g, dgdx):
        """CONLIN::UpdateVariables (CONLIN.h:91-365) for m = 1; returns (x, Newton steps)."""
        x = f64(x).copy()
        nt = C.c_int()
        check(self.L.psf_conlin_update(self.h, ptr(x), float(f), ptr(f64(dfdx)), float(g), ptr(f64(dgdx)),
                                       C.byref(nt)), allow=(PSF_OK, PSF_NOT_CONVERGED))
        return x, nt.value

    # ---------------------------------------------------------------- the whole iteration on the device
    def simp_begin(self, solver="csr_jacobi_f64", cg_eps=None, cg_itmax=None, warm_start=False, s0=None):
        pr = self.pr
        P = SimpParams()
        for name, _ in SimpParams._fields_:
            if name in pr and name not in ("optimizer", "cg_itmax", "solver", "warm_start", "heaviside",
                                            "beta_every"):
                setattr(P, name, float(pr[name]))
        P.rho0 = float(pr.get("rho0", pr["vf"]))
        P.optimizer = int(pr["optimizer"])
        P.solver = SOLVERS[solver]
        P.cg_itmax = int(pr["cg_itmax"] if cg_itmax is None else cg_itmax)
        P.cg_eps = float(pr["cg_eps"] if cg_eps is None else cg_eps)
        P.warm_start = int(bool(warm_start))
        P.heaviside = int(pr.get("heaviside", 0))
        P.beta = float(pr.get("beta", 0.5))
        P.beta_every = int(pr.get("beta_every", 40))
        P.beta_mult = float(pr.get("beta_mult", 2.0))
        self._params = P
        s0 = None if s0 is None else f64(s0)
        check(self.L.psf_simp_begin(self.h, C.byref(P), ptr(s0)))

    def simp_step(self):
        info = IterInfo()
        st = check(self.L.psf_simp_step(self.h, C.byref(info)), allow=(PSF_OK, PSF_NOT_CONVERGED, PSF_FELL_BACK))
        d = info.asdict()
        d["status"] = st
        return d

    def simp_step_host(self, s_in, s_out, rho_out=None, u_out=None):
        info = IterInfo()
        st = check(self.L.psf_simp_step_host(self.h, ptr(s_in), ptr(s_out), ptr(rho_out), ptr(u_out),
                                             C.byref(info)), allow=(PSF_OK, PSF_NOT_CONVERGED, PSF_FELL_BACK))
        d = info.asdict()
        d["status"] = st
        return d

    def fields(self):
        s, rho, dr, ds = (np.zeros(self.ne) for _ in range(4))
        u = np.zeros(self.nnodes * self.ndof)
        check(self.L.psf_simp_fields(self.h, ptr(s), ptr(rho), ptr(dr), ptr(ds), ptr(u)))
        return {"s": s, "rho": rho, "dfdrho": dr, "dfds": ds, "u": u}

    def sync(self):
        check(self.L.psf_sync(self.h))

    def export_vtk(self, path, async_=False):
        """Legacy VTK file of the current iteration (u, r, s), as the samples write it."""
        check(self.L.psf_export_vtk(self.h, str(path).encode(), int(bool(async_))))

    def export_wait(self):
        check(self.L.psf_export_wait(self.h))

    # ---------------------------------------------------------------- learned preconditioner
    def attach_learned(self, net=None, pre_mg=True, nu_pre=2, nu_post=1, use_net=True, fallback_after=0):
        """Preconditioner of the ir_learned_f32 solver: a pre-stage (one multigrid V-cycle, or
        nu_pre l1-Jacobi sweeps), the U-Net correction of the remaining residual, nu_post
        sweeps (use_net=False: the same cycle without the network)."""
        check(self.L.psf_learned_attach(self.h, None if net is None else net._h, int(bool(pre_mg)), int(nu_pre),
                                        int(nu_post), int(bool(use_net) and net is not None),
                                        int(fallback_after)))

    def learned_apply(self, r):
        """z = M(r) of the attached learned preconditioner (free-dof vectors)."""
        r = f64(r)
        z = np.zeros(self.nfree)
        check(self.L.psf_learned_apply(self.h, ptr(r), ptr(z)))
        return z

    def harvest(self, trainset, npairs, iters=None):
        """Adds npairs training pairs from the current design (see psf_learned_harvest)."""
        it = None if iters is None else np.ascontiguousarray(iters, dtype=np.int32)
        check(self.L.psf_learned_harvest(self.h, trainset._h, int(npairs), ptr(it, C.c_int),
                                         0 if it is None else len(it)))


class DeviceMMA:
    """MMA<T>(n, m, a0, a, c, d, xmin, xmax) (MMA.h:18-509) on the device for any n and
    1 <= m <= 4, per-variable bounds (psf_mma_*)."""

    def __init__(self, n, m, a0, a, c, d, xmin, xmax):
        self.L = load()
        self.n, self.m = int(n), int(m)
        h = C.c_void_p()
        xmin = f64(np.broadcast_to(np.asarray(xmin, float), (self.n,)))
        xmax = f64(np.broadcast_to(np.asarray(xmax, float), (self.n,)))
        check(self.L.psf_mma_create(self.n, self.m, float(a0), ptr(f64(a)), ptr(f64(c)), ptr(f64(d)), ptr(xmin),
                                    ptr(xmax), C.byref(h)))
        self.h = h
        self.prev = 0.0
        self.eps = 1.0e-5

    def set_parameters(self, raa0, albefa, move, asyinit, asydecr, asyincr, eps):
        self.eps = float(eps)
        check(self.L.psf_mma_set_parameters(self.h, raa0, albefa, move, asyinit, asydecr, asyincr, eps))

    def is_convergence(self, f):
        """IsConvergence (MMA.h:107-113)."""
        return abs(f - self.prev) / (f + self.prev) < self.eps

    def update(self, x, f, dfdx, g, dgdx):
        """UpdateVariables (MMA.h:116-419); returns (new x, Newton steps)."""
        x = f64(x).copy()
        nt = C.c_int()
        check(self.L.psf_mma_update_host(self.h, ptr(x), float(f), ptr(f64(dfdx)), ptr(f64(g)),
                                         ptr(f64(np.asarray(dgdx, float).reshape(-1))), C.byref(nt)),
              allow=(PSF_OK, PSF_NOT_CONVERGED))
        self.prev = float(f)
        return x, nt.value

    def close(self):
        if getattr(self, "h", None):
            self.L.psf_mma_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_simp(pr, iters, solver="csr_jacobi_f64", **kw):
    """Runs `iters` SIMP iterations on the device; returns per-iteration infos and final fields."""
    with Problem(pr) as P:
        P.setup_bc()
        P.simp_begin(solver=solver, **kw)
        infos = []
        for _ in range(iters):
            infos.append(P.simp_step())
        return infos, P.fields()
