"""The benchmark's multi-rank path on CPU (gloo, world size 2).

Replicas only: each rank processes its own images and the job's time is the
slowest rank's, so rank 0 must see the max over ranks of every timing, and
the reported throughput is world_size images per step.  The reference arm
runs on rank 0 alone; other ranks exit 0 without output.
"""
from __future__ import annotations

import argparse
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        got = bench.reduce_max(dist, [1.0 + rank, 10.0 - rank, 0.5 * rank])
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_reduce_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [2.0, 10.0, 0.5]


def test_replica_value_counts_every_rank():
    import bench
    assert bench.replica_value(1, 1_000_000, 2.0) == pytest.approx(500.0)
    assert bench.replica_value(4, 1_000_000, 2.0) == pytest.approx(2000.0)


def test_reference_arm_other_ranks_exit_quietly(capsys):
    import bench
    args = argparse.Namespace(workload="small", steps=1, warmup=3, impl="reference")
    assert bench.run_reference_arm(args, 1, 2) == 0
    assert capsys.readouterr().out == ""
