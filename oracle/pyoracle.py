"""ctypes binding of the C oracle (oracle/psf_oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference leg, as the checker.  The product library
(pansfem2_gb300) never imports it.
"""
import ctypes as C
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}

Q4_PLANE_STRAIN, Q4_HEAT, H8_SOLID = 0, 1, 2
T3_PLANE_STRAIN = 3
_SHAPE = {Q4_PLANE_STRAIN: (4, 2, 2), Q4_HEAT: (4, 1, 2), H8_SOLID: (8, 3, 3), T3_PLANE_STRAIN: (3, 2, 2)}

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)


def _lib(fast=False):
    name = "libpsf_oracle_fast.so" if fast else "libpsf_oracle.so"
    if name in _LIBS:
        return _LIBS[name]
    path = os.path.join(HERE, "_build", name)
    if not os.path.exists(path):
        raise RuntimeError(f"oracle library missing: {path} (run oracle/build.py)")
    lib = C.CDLL(path)
    lib.orc_assemble.restype = C.c_int
    lib.orc_renumber.restype = C.c_int
    for fn in ("orc_scaling_cg", "orc_cg", "orc_bicgstab", "orc_bicgstab2", "orc_ilu0_cg", "orc_scaling_bicgstab",
               "orc_ilu0_bicgstab",
               "orc_mma_update", "orc_simp_run", "orc_get_threads"):
        getattr(lib, fn).restype = C.c_int
    for fn in ("orc_true_residual", "orc_compliance_sens", "orc_oc_update", "orc_csr_get"):
        getattr(lib, fn).restype = C.c_double
    lib.orc_neighbors.restype = C.c_longlong
    lib.orc_mma_create.restype = C.c_void_p
    lib.orc_mma_update.argtypes = [C.c_void_p, dp, C.c_double, dp, dp, dp]
    lib.orc_mma_set_parameters.argtypes = [C.c_void_p] + [C.c_double] * 7
    lib.orc_mma_is_convergence.argtypes = [C.c_void_p, C.c_double]
    lib.orc_mma_destroy.argtypes = [C.c_void_p]
    lib.orc_conlin_create.restype = C.c_void_p
    lib.orc_conlin_create.argtypes = [C.c_int, C.c_int, C.c_double, dp, dp, dp, dp, dp]
    lib.orc_conlin_update.argtypes = [C.c_void_p, dp, C.c_double, dp, dp, dp]
    lib.orc_conlin_set_parameters.argtypes = [C.c_void_p, C.c_double, C.c_double]
    lib.orc_conlin_is_convergence.argtypes = [C.c_void_p, C.c_double]
    lib.orc_conlin_destroy.argtypes = [C.c_void_p]
    _LIBS[name] = lib
    return lib


def P(a, t=dp):
    return a.ctypes.data_as(t) if a is not None else None


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class CSR(C.Structure):
    _fields_ = [("rows", C.c_int), ("nnz", C.c_longlong), ("indptr", ip), ("indices", ip),
                ("data", dp)]

    def arrays(self):
        n, z = self.rows, self.nnz
        return (np.ctypeslib.as_array(self.indptr, (n + 1,)).copy(),
                np.ctypeslib.as_array(self.indices, (z,)).copy() if z else np.zeros(0, np.int32),
                np.ctypeslib.as_array(self.data, (z,)).copy() if z else np.zeros(0))


# ------------------------------------------------------------------ mesh / numbering
def q4_nodes(lx, ly, nx, ny):
    xy = np.zeros(2 * (nx + 1) * (ny + 1))
    _lib().orc_q4_nodes(C.c_double(lx), C.c_double(ly), nx, ny, P(xy))
    return xy.reshape(-1, 2)


def q4_elements(nx, ny):
    c = np.zeros(4 * nx * ny, np.int32)
    _lib().orc_q4_elements(nx, ny, P(c, ip))
    return c.reshape(-1, 4)


def h8_nodes(lx, ly, lz, nx, ny, nz):
    x = np.zeros(3 * (nx + 1) * (ny + 1) * (nz + 1))
    _lib().orc_h8_nodes(C.c_double(lx), C.c_double(ly), C.c_double(lz), nx, ny, nz, P(x))
    return x.reshape(-1, 3)


def h8_elements(nx, ny, nz):
    c = np.zeros(8 * nx * ny * nz, np.int32)
    _lib().orc_h8_elements(nx, ny, nz, P(c, ip))
    return c.reshape(-1, 8)


def renumber(nnodes, ndof, fixed_mask):
    fm = np.ascontiguousarray(fixed_mask, dtype=np.uint8)
    n2g = np.zeros(nnodes * ndof, np.int32)
    N = _lib().orc_renumber(nnodes, ndof, fm.ctypes.data_as(C.POINTER(C.c_ubyte)), P(n2g, ip))
    return n2g, N


def ke(kind, X, E, V=0.3, t=1.0):
    nen, ndof, dim = _SHAPE[kind]
    X = f64(X).reshape(-1)
    out = np.zeros((nen * ndof) ** 2)
    _lib().orc_ke(kind, P(X), C.c_double(E), C.c_double(V), C.c_double(t), P(out))
    return out.reshape(nen * ndof, nen * ndof)


def assemble(kind, conn, coords, E_e, n2g, N, V=0.3, t=1.0, ufixed=None, body=None):
    """Returns (indptr, indices, data, F) of the free x free system.  ufixed: nodal prescribed
    values (nnodes x ndof, used on the fixed dofs: F -= Ke u_fixed as Assembling.h:59-61)."""
    conn, coords, E_e, n2g = i32(conn).reshape(-1), f64(coords).reshape(-1), f64(E_e), i32(n2g)
    uf = None if ufixed is None else f64(ufixed).reshape(-1)
    ne = E_e.shape[0]
    A = CSR()
    F = np.zeros(N)
    L = _lib()
    bx, by = (0.0, 0.0) if body is None else body
    L.orc_assemble_body(kind, ne, P(conn, ip), P(coords), P(E_e), C.c_double(V), C.c_double(t),
                        P(n2g, ip), None if uf is None else P(uf), N, 0 if body is None else 1, C.c_double(bx),
                        C.c_double(by), C.byref(A), P(F))
    out = A.arrays()
    L.orc_csr_free(C.byref(A))
    return out + (F,)


def edge_loads(F, edges, coords, traction, t, n2g):
    """Uniform traction on 2-node edges (PlaneStrainSurfaceForce), added to F in edge order."""
    F = f64(F).copy()
    e = i32(edges).reshape(-1)
    _lib().orc_edge_loads(len(e) // 2, P(e, ip), P(f64(coords).reshape(-1)), C.c_double(traction[0]),
                          C.c_double(traction[1]), C.c_double(t), P(i32(n2g), ip), P(F))
    return F


def neumann(F, nodes, dofs, vals, ndof, n2g):
    nodes, dofs, vals, n2g = i32(nodes), i32(dofs), f64(vals), i32(n2g)
    _lib().orc_neumann(len(nodes), P(nodes, ip), P(dofs, ip), P(vals), ndof, P(n2g, ip), P(F))
    return F


# ------------------------------------------------------------------ solvers
def _csr_struct(indptr, indices, data):
    indptr, indices, data = i32(indptr), i32(indices), f64(data)
    A = CSR(len(indptr) - 1, len(indices), P(indptr, ip), P(indices, ip), P(data))
    A._keep = (indptr, indices, data)
    return A


def spmv(indptr, indices, data, x, fast=False):
    A = _csr_struct(indptr, indices, data)
    x = f64(x)
    y = np.zeros(A.rows)
    _lib(fast).orc_spmv(C.byref(A), P(x), P(y))
    return y


def solve(kind, indptr, indices, data, b, itmax=100000, eps=1e-10, fast=False):
    """kind in {'scaling_cg', 'cg', 'bicgstab', 'bicgstab2', 'scaling_bicgstab', 'ilu0_cg',
    'ilu0_bicgstab'}; returns (x, iters)."""
    A = _csr_struct(indptr, indices, data)
    b = f64(b)
    x = np.zeros(A.rows)
    L = _lib(fast)
    if kind in ("ilu0_cg", "ilu0_bicgstab"):
        M = CSR()
        L.orc_ilu0(C.byref(A), C.byref(M))
        it = getattr(L, "orc_" + kind)(C.byref(A), C.byref(M), P(b), itmax, C.c_double(eps), P(x))
        L.orc_csr_free(C.byref(M))
    else:
        it = getattr(L, "orc_" + kind)(C.byref(A), P(b), itmax, C.c_double(eps), P(x))
    return x, it


def ilu0(indptr, indices, data):
    A = _csr_struct(indptr, indices, data)
    M = CSR()
    L = _lib()
    L.orc_ilu0(C.byref(A), C.byref(M))
    out = M.arrays()
    L.orc_csr_free(C.byref(M))
    return out


def true_residual(indptr, indices, data, b, x):
    A = _csr_struct(indptr, indices, data)
    return _lib().orc_true_residual(C.byref(A), P(f64(b)), P(f64(x)))


# ------------------------------------------------------------------ filters / objective
def centroids(conn, coords, dim):
    conn, coords = i32(conn), f64(coords).reshape(-1)
    ne, nen = conn.shape
    cg = np.zeros(ne * dim)
    _lib().orc_centroids(ne, nen, dim, P(conn.reshape(-1), ip), P(coords), P(cg))
    return cg.reshape(ne, dim)


def neighbors(cg, R, grid=None):
    cg = f64(cg)
    ne, dim = cg.shape
    ptr = np.zeros(ne + 1, np.int32)
    idx_p, w_p = ip(), dp()
    g = i32(grid) if grid is not None else None
    L = _lib()
    cnt = L.orc_neighbors(ne, dim, P(cg.reshape(-1)), C.c_double(R), P(g, ip) if g is not None else None,
                          P(ptr, ip), C.byref(idx_p), C.byref(w_p))
    idx = np.ctypeslib.as_array(idx_p, (cnt,)).copy()
    w = np.ctypeslib.as_array(w_p, (cnt,)).copy()
    L.orc_free(C.cast(idx_p, C.c_void_p))
    L.orc_free(C.cast(w_p, C.c_void_p))
    return ptr, idx, w


def density_filter(ptr, idx, w, s):
    s = f64(s)
    out = np.zeros(len(ptr) - 1)
    _lib().orc_density_filter(len(out), P(i32(ptr), ip), P(i32(idx), ip), P(f64(w)), P(s), P(out))
    return out


def density_filter_sens(ptr, idx, w, d):
    out = np.zeros(len(ptr) - 1)
    _lib().orc_density_filter_sens(len(out), P(i32(ptr), ip), P(i32(idx), ip), P(f64(w)), P(f64(d)), P(out))
    return out


def sensitivity_filter(ptr, idx, w, s, d, mode=0):
    """SensitivityFilter (mode 0, Sigmund) / SensitivityFilter2 (mode 1, Borrvall)."""
    out = np.zeros(len(ptr) - 1)
    _lib().orc_sensitivity_filter(len(out), P(i32(ptr), ip), P(i32(idx), ip), P(f64(w)), P(f64(s)), P(f64(d)),
                                  int(mode), P(out))
    return out


def heaviside_filter(ptr, idx, w, beta, s):
    out = np.zeros(len(ptr) - 1)
    _lib().orc_heaviside_filter(len(out), P(i32(ptr), ip), P(i32(idx), ip), P(f64(w)), C.c_double(beta),
                                P(f64(s)), P(out))
    return out


def heaviside_filter_sens(ptr, idx, w, beta, s, d):
    out = np.zeros(len(ptr) - 1)
    _lib().orc_heaviside_filter_sens(len(out), P(i32(ptr), ip), P(i32(idx), ip), P(f64(w)), C.c_double(beta),
                                     P(f64(s)), P(f64(d)), P(out))
    return out


def compliance_sens(kind, conn, coords, rho, u, E1=1.0, E0=1e-9, p=3.0, V=0.3, t=1.0, scale0=1.0):
    conn, coords, rho, u = i32(conn), f64(coords).reshape(-1), f64(rho), f64(u)
    nen, ndof, dim = _SHAPE[kind]
    nnodes = coords.shape[0] // dim
    r = np.zeros(nnodes * ndof)
    d = np.zeros(len(rho))
    f = _lib().orc_compliance_sens(kind, nnodes, len(rho), P(conn.reshape(-1), ip), P(coords), P(rho),
                                   C.c_double(E1), C.c_double(E0), C.c_double(p), C.c_double(V),
                                   C.c_double(t), C.c_double(scale0), P(u), P(r), P(d))
    return f, r, d


def oc_update(x, dfdx, dgdx, ptr, idx, w, vf, iota=0.5, lmin=0.0, lmax=1e4, leps=1e-3, move=0.2,
              scale1=1.0, heaviside=0, beta=1.0):
    x = f64(x).copy()
    lam = _lib().orc_oc_update(len(x), C.c_double(iota), C.c_double(lmin), C.c_double(lmax),
                               C.c_double(leps), C.c_double(move), P(x), P(f64(dfdx)), P(f64(dgdx)),
                               P(i32(ptr), ip), P(i32(idx), ip), P(f64(w)), C.c_double(vf),
                               C.c_double(scale1), heaviside, C.c_double(beta))
    return x, lam


class MMA:
    """MMA<T> of src/Optimize/Solver/MMA.h, state kept in the C oracle."""

    def __init__(self, n, m, a0, a, c, d, xmin, xmax):
        self.n, self.m = n, m
        self._h = _lib().orc_mma_create(n, m, C.c_double(a0), P(f64(a)), P(f64(c)), P(f64(d)),
                                        P(f64(xmin)), P(f64(xmax)))

    def set_parameters(self, raa0, albefa, move, asyinit, asydecr, asyincr, eps):
        _lib().orc_mma_set_parameters(self._h, raa0, albefa, move, asyinit, asydecr, asyincr, eps)

    def is_convergence(self, f):
        return bool(_lib().orc_mma_is_convergence(self._h, f))

    def update(self, x, f, dfdx, g, dgdx):
        x = f64(x).copy()
        newton = _lib().orc_mma_update(self._h, P(x), f, P(f64(dfdx)), P(f64(g)), P(f64(dgdx).reshape(-1)))
        return x, newton

    def __del__(self):
        try:
            _lib().orc_mma_destroy(self._h)
        except Exception:
            pass


class CONLIN:
    """CONLIN<T> of src/Optimize/Solver/CONLIN.h, state kept in the C oracle."""

    def __init__(self, n, m, a0, a, c, d, xmin, xmax):
        self.n, self.m = n, m
        self._h = _lib().orc_conlin_create(n, m, a0, P(f64(a)), P(f64(c)), P(f64(d)), P(f64(xmin)),
                                           P(f64(xmax)))

    def set_parameters(self, move, eps):
        _lib().orc_conlin_set_parameters(self._h, move, eps)

    def is_convergence(self, f):
        return bool(_lib().orc_conlin_is_convergence(self._h, f))

    def update(self, x, f, dfdx, g, dgdx):
        x = f64(x).copy()
        newton = _lib().orc_conlin_update(self._h, P(x), f, P(f64(dfdx)), P(f64(g)), P(f64(dgdx).reshape(-1)))
        return x, newton

    def __del__(self):
        try:
            _lib().orc_conlin_destroy(self._h)
        except Exception:
            pass


# ------------------------------------------------------------------ SIMP loop
class SimpCfg(C.Structure):
    _fields_ = [("kind", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
                ("V", C.c_double), ("t", C.c_double), ("E1", C.c_double), ("E0", C.c_double),
                ("p", C.c_double), ("vf", C.c_double), ("R", C.c_double), ("scale0", C.c_double),
                ("scale1", C.c_double), ("rho0", C.c_double), ("optimizer", C.c_int),
                ("oc_iota", C.c_double), ("oc_lmin", C.c_double), ("oc_lmax", C.c_double),
                ("oc_leps", C.c_double), ("oc_move", C.c_double),
                ("mma_raa0", C.c_double), ("mma_albefa", C.c_double), ("mma_move", C.c_double),
                ("mma_asyinit", C.c_double), ("mma_asydecr", C.c_double), ("mma_asyincr", C.c_double),
                ("mma_eps", C.c_double), ("mma_a0", C.c_double), ("mma_c", C.c_double),
                ("mma_d", C.c_double), ("mma_xmin", C.c_double), ("mma_xmax", C.c_double),
                ("cg_itmax", C.c_int), ("cg_eps", C.c_double), ("heaviside", C.c_int),
                ("nfix", C.c_int), ("fix_node", ip), ("fix_dof", ip),
                ("nload", C.c_int), ("load_node", ip), ("load_dof", ip), ("load_val", dp)]


class SimpOut(C.Structure):
    _fields_ = [("f", dp), ("g", dp), ("lambda_", dp), ("cg_iters", ip), ("mma_newton", ip),
                ("true_res", dp), ("rho", dp), ("dfdrho", dp), ("dfds", dp), ("s_after", dp),
                ("u", dp), ("s_final", dp), ("phase_seconds", dp)]


def simp_run(problem, iters, fields=False, fast=False, stop_on_convergence=False):
    """problem: a pansfem2-style dict (see tests/problems.py).  Returns a dict of arrays."""
    pr = problem
    kind = pr["kind"]
    nen, ndof, dim = _SHAPE[kind]
    nx, ny, nz = pr["nx"], pr["ny"], pr.get("nz", 0)
    ne = nx * ny * (nz if kind == H8_SOLID else 1)
    nnodes = (nx + 1) * (ny + 1) * ((nz + 1) if kind == H8_SOLID else 1)
    keep = []

    def arr(a, t):
        a = i32(a) if t is ip else f64(a)
        keep.append(a)
        return P(a, t)

    cfg = SimpCfg()
    for k in ("kind", "nx", "ny", "nz"):
        setattr(cfg, k, int(pr.get(k, 0)))
    for k, dflt in (("lx", nx), ("ly", ny), ("lz", nz), ("V", 0.3), ("t", 1.0), ("E1", 1.0),
                    ("E0", 1e-9), ("p", 3.0), ("vf", 0.5), ("R", 1.5), ("scale0", 1.0),
                    ("scale1", 1.0), ("oc_iota", 0.5), ("oc_lmin", 0.0), ("oc_lmax", 1e4),
                    ("oc_leps", 1e-3), ("oc_move", 0.2), ("mma_raa0", 1e-5), ("mma_albefa", 0.1),
                    ("mma_move", 0.2), ("mma_asyinit", 0.5), ("mma_asydecr", 0.7),
                    ("mma_asyincr", 1.2), ("mma_eps", 1e-6), ("mma_a0", 1.0), ("mma_c", 1e4),
                    ("mma_d", 0.0), ("mma_xmin", 0.01), ("mma_xmax", 1.0), ("cg_eps", 1e-10)):
        setattr(cfg, k, float(pr.get(k, dflt)))
    cfg.rho0 = float(pr.get("rho0", cfg.vf))
    cfg.optimizer = int(pr.get("optimizer", 0))
    cfg.cg_itmax = int(pr.get("cg_itmax", 100000))
    cfg.heaviside = int(pr.get("heaviside", 0))
    cfg.nfix = len(pr["fix_node"])
    cfg.fix_node, cfg.fix_dof = arr(pr["fix_node"], ip), arr(pr["fix_dof"], ip)
    cfg.nload = len(pr["load_node"])
    cfg.load_node, cfg.load_dof = arr(pr["load_node"], ip), arr(pr["load_dof"], ip)
    cfg.load_val = arr(pr["load_val"], dp)

    res = {"f": np.zeros(iters), "g": np.zeros(iters), "lambda": np.zeros(iters),
           "cg_iters": np.zeros(iters, np.int32), "mma_newton": np.zeros(iters, np.int32),
           "true_res": np.zeros(iters), "s_final": np.zeros(ne), "phase_seconds": np.zeros(8)}
    if fields:
        for k, n in (("rho", ne), ("dfdrho", ne), ("dfds", ne), ("s_after", ne), ("u", nnodes * ndof)):
            res[k] = np.zeros(iters * n)
    out = SimpOut()
    out.f, out.g, out.lambda_ = P(res["f"]), P(res["g"]), P(res["lambda"])
    out.cg_iters, out.mma_newton = P(res["cg_iters"], ip), P(res["mma_newton"], ip)
    out.true_res, out.s_final, out.phase_seconds = P(res["true_res"]), P(res["s_final"]), P(res["phase_seconds"])
    if fields:
        out.rho, out.dfdrho, out.dfds = P(res["rho"]), P(res["dfdrho"]), P(res["dfds"])
        out.s_after, out.u = P(res["s_after"]), P(res["u"])
    done = _lib(fast).orc_simp_run(C.byref(cfg), iters, int(stop_on_convergence), C.byref(out))
    res["done"] = done
    if fields:
        for k, n in (("rho", ne), ("dfdrho", ne), ("dfds", ne), ("s_after", ne), ("u", nnodes * ndof)):
            res[k] = res[k].reshape(iters, n)
    return res


def set_threads(n, fast=True):
    _lib(fast).orc_set_threads(int(n))


def get_threads(fast=True):
    return _lib(fast).orc_get_threads()


# ------------------------------------------------------------------ dump reader
def read_dump(path):
    """Reads the [namelen][name][type][count][data] container written by ref_driver."""
    out = {}
    with open(path, "rb") as fh:
        buf = fh.read()
    o = 0
    while o < len(buf):
        (nl,) = struct.unpack_from("<i", buf, o); o += 4
        name = buf[o:o + nl].decode(); o += nl
        typ, cnt = struct.unpack_from("<iq", buf, o); o += 12
        dt = np.float64 if typ == 0 else np.int32
        n = cnt * np.dtype(dt).itemsize
        out[name] = np.frombuffer(buf[o:o + n], dtype=dt).copy(); o += n
    return out


# ---------------------------------------------------------------- U-Net oracle
_unet = None


def _unet_lib():
    global _unet
    if _unet is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "libunet_oracle.so")
        if not os.path.exists(path):
            from oracle import build as _b
            _b.build()
        lib = C.CDLL(path)
        lib.uo_nparams.restype = C.c_int
        lib.uo_loss_grad.restype = C.c_double
        lib.uo_loss_grad.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        _unet = lib
    return _unet


def unet_nparams(c0=16):
    return int(_unet_lib().uo_nparams(c0))


def unet_loss_grad(params, inp, target, mask=None, c0=16, bf16=True, want_grad=True):
    """Loss, output [B,H,W,2] and parameter gradient of the U-Net oracle.
    inp: float32 [B,H,W,8]; target, mask: float32 [B,H,W,2]."""
    params = np.ascontiguousarray(params, dtype=np.float32)
    inp = np.ascontiguousarray(inp, dtype=np.float32)
    target = np.ascontiguousarray(target, dtype=np.float32)
    B, H, W, _ = inp.shape
    out = np.zeros((B, H, W, 2), np.float32)
    grad = np.zeros(params.size, np.float32) if want_grad else None
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    loss = _unet_lib().uo_loss_grad(params.ctypes.data, c0, B, H, W, inp.ctypes.data, target.ctypes.data,
                                    None if m is None else m.ctypes.data, int(bf16), out.ctypes.data,
                                    None if grad is None else grad.ctypes.data)
    return loss, out, grad
