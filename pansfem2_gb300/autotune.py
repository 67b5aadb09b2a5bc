"""Launch-shape autotuner.

Times each candidate launch shape on the workload itself (CUDA-event device
time of a few real iterations after warm-up) and keeps the fastest.  Results
are cached per process and, when PSF_TUNE_CACHE names a JSON file, across
processes, keyed by the GPU name and a signature of the workload.

Tuned today:
  batch          threads per CTA (256 / 512) and CTAs per instance (a thread-block
                 cluster of 1, 2, 4 or 8) of the batched heat-conduction SIMP.  More
                 CTAs per instance shorten the largest instances' critical path
                 (one SM's bandwidth and FP64 rate bound a lone CTA); fewer leave
                 room for more instances at once.
  pcg            lanes per CSR row (1: one lane per row on the sliced copy), threads per block and blocks per SM of the
                 persistent FP64 CSR PCG (psf_set_launch_shape PSF_KERNEL_PCG_CSR),
                 timed on the Problem's own assembled system.
  opt            blocks per SM of the persistent OC / MMA / CONLIN kernels
                 (PSF_KERNEL_OPT), timed on one update of the Problem's design.
"""
import hashlib
import json
import os

import numpy as np

_CACHE = {}


def _gpu_name():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def _load():
    path = os.environ.get("PSF_TUNE_CACHE")
    if path and os.path.exists(path):
        try:
            with open(path) as fh:
                _CACHE.update(json.load(fh))
        except Exception:
            pass


def _store():
    path = os.environ.get("PSF_TUNE_CACHE")
    if path:
        try:
            with open(path, "w") as fh:
                json.dump(_CACHE, fh, indent=1, sort_keys=True)
        except Exception:
            pass


def _key(kind, sig):
    h = hashlib.sha1(json.dumps(sig, sort_keys=True).encode()).hexdigest()[:16]
    return f"{kind}|{_gpu_name()}|{h}"


def pick(key, candidates, timer, log=None):
    """The candidate with the least time(candidate) (None = not runnable), cached under key:
    a cached key returns its choice without timing anything.  Returns (best, {str: seconds})."""
    _load()
    if key in _CACHE:
        ent = _CACHE[key]
        return tuple(ent["best"]), ent["times"]
    times = {}
    for cand in candidates:
        try:
            t = timer(cand)
        except Exception as e:   # a shape the device cannot launch is skipped
            if log:
                log(f"autotune {key} {cand}: {e}")
            continue
        if t is not None:
            times["x".join(str(v) for v in cand)] = float(t)
    if not times:
        raise RuntimeError(f"autotune {key}: no candidate ran")
    best = min(times, key=times.get)
    _CACHE[key] = {"best": [int(v) for v in best.split("x")], "times": times}
    _store()
    return tuple(_CACHE[key]["best"]), times


PCG_CANDIDATES = ((1, 256, 4), (1, 512, 2), (1, 1024, 1), (4, 512, 2), (4, 1024, 1), (8, 1024, 1))


def tune_pcg(prob, candidates=PCG_CANDIDATES, iters=300, log=None):
    """(lanes per row, threads, blocks per SM) of the FP64 CSR PCG for this Problem (its system
    assembled at the uniform design vf): device time per iteration of `iters` fixed iterations;
    the best shape is set on the Problem and returned with the timings."""
    from ._lib import PSF_KERNEL_PCG_CSR
    pr = prob.pr
    prob.assemble(np.full(prob.ne, float(pr.get("vf", 0.5)) ** float(pr.get("p", 3.0))))

    def timer(c):
        prob.set_launch_shape(PSF_KERNEL_PCG_CSR, *c)
        prob.solve("csr_jacobi_f64", itmax=iters, eps=1e-30)   # warm-up
        _, info = prob.solve("csr_jacobi_f64", itmax=iters, eps=1e-30)
        return info["kernel_seconds"] / max(1, info["iterations"])

    key = _key("pcg", {"kind": pr["kind"], "nx": pr["nx"], "ny": pr["ny"], "nz": pr.get("nz", 0),
                       "cands": [list(c) for c in candidates]})
    best, times = pick(key, candidates, timer, log)
    prob.set_launch_shape(PSF_KERNEL_PCG_CSR, *best)
    return best, times


def tune_opt(pr, candidates=((1,), (2,), (3,), (4,)), solver="ir_mg_f32", log=None):
    """Blocks per SM of the persistent OC / MMA / CONLIN kernels for problem dict pr: the device
    time of the update phase of SIMP iteration 1 (a fresh Problem per candidate).  Returns
    ((blocks per SM,), timings); set it with Problem.set_launch_shape(PSF_KERNEL_OPT, 0, 256, bps)."""
    from . import api
    from ._lib import PSF_KERNEL_OPT

    def timer(c):
        with api.Problem(pr) as P:
            P.set_launch_shape(PSF_KERNEL_OPT, 0, 256, c[0])
            P.setup_bc()
            P.simp_begin(solver=solver, cg_eps=1e-8, warm_start=True)
            P.simp_step()
            return P.simp_step()["phase_seconds"][5]

    key = _key("opt", {"kind": pr["kind"], "nx": pr["nx"], "ny": pr["ny"], "nz": pr.get("nz", 0),
                       "opt": int(pr.get("optimizer", 0)), "cands": [list(c) for c in candidates]})
    return pick(key, candidates, timer, log)


def tune_batch(instances, candidates=((256, 1), (512, 1), (256, 4), (512, 2), (512, 4), (512, 8)), iters=2,
               warmup=1, cg_eps=1e-8, log=None):
    """(threads per CTA, CTAs per instance) for HeatBatch(instances): the candidate with
    the least device time for `iters` SIMP iterations after `warmup` iterations (each
    candidate starts from the same initial design).  Returns ((threads, cluster),
    {"threads x cluster": seconds})."""
    from .batch import HeatBatch
    _load()
    key = _key("batch", {"inst": [(d["side"], d["edge"], d["patch_w"], d["patch_i0"], round(d["vf"], 6))
                                  for d in instances], "eps": cg_eps, "cands": [list(c) for c in candidates]})
    if key in _CACHE:
        ent = _CACHE[key]
        return tuple(ent["best"]), ent["times"]
    times = {}
    for t, c in candidates:
        try:
            with HeatBatch(instances, threads=t, cluster=c) as B:
                B.begin(cg_eps=cg_eps)
                if warmup:
                    B.step(warmup)
                sec = B.step(iters)
        except Exception as e:   # a shape the device cannot launch is skipped
            if log:
                log(f"autotune batch {t}x{c}: {e}")
            continue
        times[f"{t}x{c}"] = sec
        if log:
            log(f"autotune batch {t}x{c}: {sec * 1e3:.2f} ms for {iters} iterations")
    best = min(times, key=times.get)
    bt, bc = (int(v) for v in best.split("x"))
    _CACHE[key] = {"best": [bt, bc], "times": times}
    _store()
    return (bt, bc), times
