"""Host-side pieces of bench.py that need no GPU: the CPU path's
size-scaling points (one oracle run per size, written as JSON lines)."""
import json
import os
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def test_cpu_scaling_child_writes_one_point_per_size(tmp_path, monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setattr(bench, "CPU_SCALING_SIZES", (12, 20))
    path = str(tmp_path / "points.jsonl")
    assert bench.cpu_scaling_child(path, 0.04) == 0
    rows = [json.loads(x) for x in open(path)]
    assert [r["edge"] for r in rows] == [12, 20]
    for r in rows:
        assert r["voxels"] == r["edge"] ** 3 and r["seconds"] > 0
        assert r["voxels_per_s"] == r["voxels"] / r["seconds"]
