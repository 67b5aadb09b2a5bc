"""The autotuner's choice and cache (no GPU: a stand-in timer): the fastest candidate wins,
unrunnable candidates are skipped, a cached key returns its choice without timing anything,
and the cache file written by one process is read by the next."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pick_times_once_then_reuses(tmp_path, monkeypatch):
    from pansfem2_gb300 import autotune as T
    monkeypatch.setenv("PSF_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(T, "_CACHE", {})
    calls = []

    def timer(c):
        calls.append(c)
        if c == (8, 256, 4):
            raise RuntimeError("does not fit")
        return {(4, 256, 4): 3.0, (4, 1024, 1): 1.5, (16, 1024, 1): 2.0}[c]

    cands = ((4, 256, 4), (8, 256, 4), (4, 1024, 1), (16, 1024, 1))
    best, times = T.pick("pcg|test", cands, timer)
    assert best == (4, 1024, 1) and set(times) == {"4x256x4", "4x1024x1", "16x1024x1"}
    n = len(calls)
    best2, _ = T.pick("pcg|test", cands, timer)
    assert best2 == best and len(calls) == n   # reused, nothing timed
    saved = json.load(open(tmp_path / "tune.json"))
    assert saved["pcg|test"]["best"] == [4, 1024, 1]
    # a fresh process reads the cache file and times nothing
    code = ("import sys; sys.path.insert(0, %r); from pansfem2_gb300 import autotune as T\n"
            "def t(c): raise SystemExit('timed')\n"
            "print(T.pick('pcg|test', ((1, 1, 1),), t)[0])" % ROOT)
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True,
                         env=dict(os.environ, PSF_TUNE_CACHE=str(tmp_path / "tune.json")))
    assert out.returncode == 0 and out.stdout.strip() == "(4, 1024, 1)", out.stderr


def test_pick_with_nothing_runnable_raises(monkeypatch):
    from pansfem2_gb300 import autotune as T
    monkeypatch.delenv("PSF_TUNE_CACHE", raising=False)
    monkeypatch.setattr(T, "_CACHE", {})

    def timer(c):
        raise RuntimeError("no")

    with pytest.raises(RuntimeError):
        T.pick("x|y", ((1,),), timer)
