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
"""
import hashlib
import json
import os

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
