"""Multi-process host logic on CPU (gloo, world size 2).

The solve does not shard: N GPUs run N independent replicas, which only meet
at barriers and agree on the slowest rank's time (kamsta_gb300.replicas).
These tests run that coordination, and the bench's reference arm under
torchrun, with two CPU processes.
"""
import json
import multiprocessing as mp
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    from kamsta_gb300.replicas import Replicas
    r = Replicas()
    r.barrier()
    mx = r.max(10.0 + rank)
    sm = r.sum(1.0 + rank)
    r.barrier()
    r.close()
    q.put((rank, mx, sm))


def test_replicas_max_and_sum_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 11.0, 3.0), (1, 11.0, 3.0)]


def test_single_process_replicas_are_identity():
    sys.path.insert(0, ROOT)
    from kamsta_gb300.replicas import Replicas
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK") if k in os.environ}
    try:
        r = Replicas()
        assert (r.world, r.rank) == (1, 0)
        assert r.max(3.5) == 3.5 and r.sum(2.0) == 2.0
        r.barrier()
        r.close()
    finally:
        os.environ.update(env)


def test_bench_reference_arm_under_torchrun_two_ranks():
    """Rank 0 alone times the reference's CPU code (its own build, or the
    oracle's restatement where that cannot be built) and prints one JSON
    line; the other rank exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
           "--sample-log-n", "10", "--sample-log-m", "13"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["value"] > 0
    assert d["config"]["host"]["logical_cpus"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0


def test_workload_mix_is_seeded_and_in_range():
    sys.path.insert(0, ROOT)
    from kamsta_gb300 import workloads as W
    a = W.mixed_specs(512, 7)
    b = W.mixed_specs(512, 7)
    assert a == b
    assert all(256 <= s.n <= (1 << 20) and 4 <= s.avg_degree <= 32 for s in a)
    assert [s.family for s in a[:4]] == ["gnm", "rgg2d", "gnm", "rgg2d"]
    assert len({s.seed for s in a}) == len(a)
    p = W.percentiles([1.0] * 98 + [5.0, 9.0])
    assert p["p50_ms"] == 1.0 and 1.0 < p["p99_ms"] <= 9.0
