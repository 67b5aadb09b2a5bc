"""The N-rank path of bench.py on CPU, with the gloo backend and two ranks on 127.0.0.1.

One problem does not shard (replicas only): each rank runs its own copy of the workload, the
ranks meet at barriers around the timed region, and the job's time is the slowest rank's.
These tests check that reduction (bench.max_over_ranks) across real processes, the rank
seeding of the batch workload, and that the reference arm under torchrun prints one line from
rank 0 while the other ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r took (1 + r) s for the device leg and (5 - r) s end to end
    got = bench.max_over_ranks([1.0 + rank, 5.0 - rank], world)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got))


def test_max_over_ranks_with_gloo():
    import multiprocessing as mp
    torch = pytest.importorskip("torch")  # noqa: F841
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 5.0]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3, 4.5], 1) == [3.0, 4.5]


def test_batch_replicas_are_seeded_by_rank():
    from pansfem2_gb300 import problems as PB
    a, b = PB.heat_batch(8, seed=0), PB.heat_batch(8, seed=1)
    assert [d["side"] for d in a] == [d["side"] for d in PB.heat_batch(8, seed=0)]
    assert [(d["side"], d["vf"]) for d in a] != [(d["side"], d["vf"]) for d in b]


def test_reference_arm_under_torchrun_prints_one_line():
    pytest.importorskip("torch")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--nx", "24", "--ny", "12"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"

