"""Explicit (unstructured) meshes: the reference's general assembly path on the device.

A mesh is node coordinates plus element connectivity (T3 or Q4 plane strain, Q4 heat, H8
solid), as the reference's ImportFromCSV.h reads them or sample_planestrain.cpp writes them
out.  FemMesh assembles the same CSR system (numbering, pattern, values, loads) the
reference's SetDirichlet / Renumbering / Assembling / CSR(LILCSR&) sequence builds, bit for
bit, solves it with ScalingCG or CG and forms the reaction forces.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, f64, ptr

T3_PLANE_STRAIN = 3
_NEN = {0: 4, 1: 4, 2: 8, 3: 3}
_NDOF = {0: 2, 1: 1, 2: 3, 3: 2}
_DIM = {0: 2, 1: 2, 2: 3, 3: 2}


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


class FemMesh:
    def __init__(self, kind, coords, conn):
        self.L = _lib.load()
        self.kind = int(kind)
        self.coords = f64(np.asarray(coords, float).reshape(-1, _DIM[self.kind]))
        self.conn = _i32(np.asarray(conn).reshape(-1, _NEN[self.kind]))
        self.nnodes, self.ne = len(self.coords), len(self.conn)
        self.ndof = _NDOF[self.kind]
        self.nfree = 0
        self.nnz = 0
        h = C.c_void_p()
        check(self.L.psf_fem_create(self.kind, self.nnodes, ptr(self.coords), self.ne, _NEN[self.kind],
                                    self.conn.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.psf_fem_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_dirichlet(self, node, dof, value=None):
        node, dof = _i32(node), _i32(dof)
        nf = C.c_int()
        v = None if value is None else f64(value)
        check(self.L.psf_fem_set_dirichlet(self.h, len(node), node.ctypes.data_as(C.POINTER(C.c_int32)),
                                           dof.ctypes.data_as(C.POINTER(C.c_int32)), ptr(v), C.byref(nf)))
        self.nfree = nf.value
        return self.nfree

    def set_loads(self, node, dof, value):
        node, dof, value = _i32(node), _i32(dof), f64(value)
        check(self.L.psf_fem_set_loads(self.h, len(node), node.ctypes.data_as(C.POINTER(C.c_int32)),
                                       dof.ctypes.data_as(C.POINTER(C.c_int32)), ptr(value)))

    def set_body_force(self, fx, fy):
        check(self.L.psf_fem_set_body_force(self.h, float(fx), float(fy)))

    def set_edge_loads(self, edges, tx, ty):
        edges = _i32(np.asarray(edges).reshape(-1, 2))
        check(self.L.psf_fem_set_edge_loads(self.h, len(edges), edges.ctypes.data_as(C.POINTER(C.c_int32)),
                                            float(tx), float(ty)))

    def assemble(self, E, V=0.3, t=1.0):
        E = f64(np.broadcast_to(np.asarray(E, float), (self.ne,)).copy())
        nnz = C.c_longlong()
        check(self.L.psf_fem_assemble(self.h, ptr(E), float(V), float(t), C.byref(nnz)))
        self.nnz = nnz.value
        return self.nnz

    def timings(self):
        """Device milliseconds of the last assemble: element matrices, pattern, values."""
        t = [C.c_double() for _ in range(3)]
        check(self.L.psf_fem_timings(self.h, *[C.byref(x) for x in t]))
        return [x.value for x in t]

    def system(self):
        """(n2g, indptr, indices, data, F) of the assembled free-dof system."""
        n2g = np.zeros(self.nnodes * self.ndof, np.int32)
        ip = np.zeros(self.nfree + 1, np.int32)
        ix = np.zeros(max(self.nnz, 1), np.int32)
        d = np.zeros(max(self.nnz, 1))
        F = np.zeros(max(self.nfree, 1))
        P32 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
        check(self.L.psf_fem_get_system(self.h, P32(n2g), P32(ip), P32(ix), ptr(d), ptr(F)))
        return n2g, ip, ix[:self.nnz], d[:self.nnz], F[:self.nfree]

    def solve(self, solver="scaling_cg", itmax=100000, eps=1e-10):
        """Nodal solution (nnodes x ndof) with ScalingCG ("scaling_cg") or CG ("cg")."""
        code = {"scaling_cg": 0, "cg": 4}[solver]
        u = np.zeros(self.nnodes * self.ndof)
        info = _lib.SolveInfo()
        st = check(self.L.psf_fem_solve(self.h, code, int(itmax), float(eps), ptr(u), C.byref(info)),
                   allow=(0, 1))
        d = info.asdict()
        d["status"] = st
        return u, d

    def reaction(self, u):
        u = f64(u)
        r = np.zeros(self.nnodes * self.ndof)
        check(self.L.psf_fem_reaction(self.h, ptr(u), ptr(r)))
        return r
