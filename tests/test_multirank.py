"""The multi-rank host path of bench.py (replicas: one independent volume
per rank, no collective on the data path) with world size 2 on CPU over
gloo: the timing is the slowest rank's, the throughput counts every rank's
voxels, and the reference arm runs on rank 0 only."""
import argparse
import os
import socket
import sys

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    own_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    ms = bench.max_over_ranks(own_ms, dist)
    value = bench.replica_throughput(world, 1000, 4, ms)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, ms, value))


def test_two_ranks_over_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in res:
        assert ms == 150.0  # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 1000 * 4 / 0.150)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = argparse.Namespace(steps=1, warmup=1, t=0.04)
    assert bench.run_reference(args) == 0  # returns at once, no work
