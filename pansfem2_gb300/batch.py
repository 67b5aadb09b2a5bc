"""Batched heat-conduction SIMP (psf_batch_*): many independent heat-sink
instances of uneven size advanced together, one CTA per instance, one SIMP
iteration of all of them per CUDA-graph replay.  No counterpart in the
reference, whose samples run one problem per process."""
import ctypes as C

import numpy as np

from . import _lib as L
from . import problems as PB

RESULT_FIELDS = ("f", "g", "lambda", "iters", "res", "conv", "passes", "bisect", "f_prev", "done")


class HeatBatch:
    def __init__(self, instances, threads=512, cluster=1):
        """instances: dicts with side, edge, patch_w, patch_i0, vf (problems.heat_batch);
        a team of `cluster` CTAs (a thread-block cluster) of `threads` threads per instance."""
        self.inst = [dict(d) for d in instances]
        n = len(self.inst)
        arr = lambda k, t: np.ascontiguousarray([d[k] for d in self.inst], dtype=t)  # noqa: E731
        self._keep = [arr("side", np.int32), arr("edge", np.int32), arr("patch_w", np.int32),
                      arr("patch_i0", np.int32), arr("vf", np.float64)]
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
        h = C.c_void_p()
        L.check(L.load().psf_batch_create(n, ip(self._keep[0]), ip(self._keep[1]), ip(self._keep[2]),
                                          ip(self._keep[3]), L.ptr(self._keep[4]), int(threads), int(cluster),
                                          C.byref(h)))
        self._h, self.n = h, n

    def close(self):
        if self._h:
            L.load().psf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def begin(self, cg_eps=1e-8, cg_itmax=2000, warm_start=True, **kw):
        """Shared parameters: those of problems.heatsink_q4 (k0 = E1 = 1, kmin = E0 = 1e-3,
        p = 3, R = 1.5, OC) unless overridden."""
        pr = PB.heatsink_q4(8, 8, **kw)
        P = L.SimpParams()
        for name, _ in L.SimpParams._fields_:
            if name in pr and name not in ("optimizer", "cg_itmax", "solver", "warm_start", "heaviside",
                                            "beta_every"):
                setattr(P, name, float(pr[name]))
        P.optimizer = 0
        P.solver = L.SOLVERS["ir_mg_f32"]
        P.cg_itmax = int(cg_itmax)
        P.cg_eps = float(cg_eps)
        P.warm_start = int(bool(warm_start))
        self._params = P
        L.check(L.load().psf_batch_begin(self._h, C.byref(P)))

    def step(self, iters=1):
        """iters SIMP iterations of every instance; returns device seconds."""
        t = C.c_double()
        L.check(L.load().psf_batch_step(self._h, int(iters), C.byref(t)))
        return t.value

    def profile(self):
        """One SIMP iteration without the graph: device seconds per phase."""
        out = np.zeros(4)
        L.check(L.load().psf_batch_profile(self._h, L.ptr(out)))
        return dict(zip(("filter_moduli", "solve", "sens", "oc"), out))

    def results(self):
        out = np.zeros((self.n, len(RESULT_FIELDS)))
        L.check(L.load().psf_batch_results(self._h, L.ptr(out)))
        return {k: out[:, i] for i, k in enumerate(RESULT_FIELDS)}

    def fields(self, k):
        side = self.inst[k]["side"]
        s, rho = np.zeros(side * side), np.zeros(side * side)
        T = np.zeros((side + 1) ** 2)
        L.check(L.load().psf_batch_fields(self._h, int(k), L.ptr(s), L.ptr(rho), L.ptr(T)))
        return {"s": s, "rho": rho, "T": T}

    def problem(self, k, **kw):
        """The instance as a single-problem dict (problems.heatsink_q4)."""
        d = self.inst[k]
        return PB.heatsink_q4(d["side"], d["side"], patch_w=d["patch_w"], patch_i0=d["patch_i0"], edge=d["edge"],
                              vf=d["vf"], **kw)
