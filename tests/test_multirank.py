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


# ---- whole volumes across ranks (the batched path on several GPUs) ---------

def _csg_set():
    from voxel_ma_gb300 import volumes
    return [volumes.csg(700 + i, 10, 26) for i in range(10)]


def _volume_digest(r):
    import hashlib
    import numpy as np
    h = hashlib.sha256()
    for k in ("rem_vts", "rem_edges", "rem_tris"):
        h.update(np.ascontiguousarray(r[k]).tobytes())
    for k in ("keep_v", "keep_e", "keep_f"):
        h.update(np.ascontiguousarray(r["thin"][k]).tobytes())
    return h.hexdigest()


def _partition_rank_main(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import oracle
    from voxel_ma_gb300 import api
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    vols = _csg_set()
    part = api.partition_volumes([v.size for v in vols], world)
    mine = {i: _volume_digest(oracle.run_plain(vols[i], 0.04)) for i in range(len(vols)) if part[i] == rank}
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    dist.barrier()
    dist.destroy_process_group()
    out.put((rank, [int(p) for p in part], gathered))


def test_volumes_partitioned_across_two_gloo_ranks():
    """Each rank takes its share of a CSG volume set (vc_partition_volumes)
    and runs it; the union gathered over gloo equals one process running
    every volume, and every volume ran exactly once."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import oracle
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_partition_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    vols = _csg_set()
    single = {i: _volume_digest(oracle.run_plain(v, 0.04)) for i, v in enumerate(vols)}
    (r0, part0, g0), (r1, part1, g1) = res
    assert part0 == part1 and set(part0) == {0, 1}
    union = {}
    for d in g0:
        for i, h in d.items():
            assert i not in union  # no volume ran twice
            union[i] = h
    assert union == single
    assert g0 == g1


def test_partition_rule():
    import numpy as np

    from voxel_ma_gb300 import api
    rng = np.random.default_rng(1)
    for nparts in (1, 2, 3, 8):
        vox = np.exp(rng.uniform(np.log(32 ** 3), np.log(192 ** 3), 256)).astype(np.int64)
        part = api.partition_volumes(vox, nparts)
        assert part.min() >= 0 and part.max() < nparts
        load = np.bincount(part, weights=vox, minlength=nparts)
        assert load.max() - load.min() <= vox.max()  # greedy largest-first bound
    assert list(api.partition_volumes([5, 9, 1, 9], 2)) == [0, 0, 1, 1]
