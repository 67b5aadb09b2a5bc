"""Launch-shape autotuner.

Times each candidate launch shape on the workload itself (CUDA-event device
time of a few real iterations after warm-up) and keeps the fastest.  Results
are cached per process and, when PSF_TUNE_CACHE names a JSON file, across
processes, keyed by the GPU name and a signature of the workload.

Tuned today:
  batch_threads  threads per CTA of the batched heat-conduction SIMP (one CTA
                 per instance): 128 / 256 / 512 (the kernels' launch bound).  Fewer threads leave
                 room for more CTAs per SM (small instances); more threads
                 shorten the largest instances' critical path.
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


def tune_batch_threads(instances, candidates=(128, 256, 512), iters=2, warmup=1, cg_eps=1e-8, log=None):
    """Threads per CTA for HeatBatch(instances): the candidate with the least device
    time for `iters` SIMP iterations after `warmup` iterations (each candidate starts
    from the same initial design).  Returns (threads, {threads: seconds})."""
    from .batch import HeatBatch
    _load()
    key = _key("batch_threads", {"inst": [(d["side"], d["edge"], d["patch_w"], d["patch_i0"], round(d["vf"], 6))
                                          for d in instances], "eps": cg_eps, "cands": list(candidates)})
    if key in _CACHE:
        ent = _CACHE[key]
        return ent["best"], {int(k): v for k, v in ent["times"].items()}
    times = {}
    for t in candidates:
        with HeatBatch(instances, threads=t) as B:
            B.begin(cg_eps=cg_eps)
            if warmup:
                B.step(warmup)
            times[t] = B.step(iters)
        if log:
            log(f"autotune batch_threads {t}: {times[t] * 1e3:.2f} ms for {iters} iterations")
    best = min(times, key=times.get)
    _CACHE[key] = {"best": best, "times": times}
    _store()
    return best, times
