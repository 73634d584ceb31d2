"""The request loop's batching rule (vc_plan_batches, the rule the server's
workers apply), checked on the host against a plain restatement."""
import numpy as np
import pytest

from voxel_ma_gb300 import _lib, api


def _restated(voxels, t, share, bpv, max_batch):
    out, b, count, total, tb = [], -1, 0, 0.0, None
    for v, tt in zip(voxels, t):
        e = bpv * v
        if v <= 0 or e > share:
            out.append(-1)
            continue
        if b < 0 or count >= max_batch or tt != tb or total + e > share:
            b, count, total, tb = b + 1, 0, 0.0, tt
        out.append(b)
        count += 1
        total += e
    return np.array(out, np.int32)


def test_rule_matches_restatement_on_random_streams():
    rng = np.random.default_rng(0)
    for _ in range(50):
        n = int(rng.integers(0, 200))
        vox = np.exp(rng.uniform(np.log(32 ** 3), np.log(384 ** 3), n)).astype(np.int64)
        t = rng.choice([0.04, 0.04, 0.04, 0.1], n)
        share = int(rng.uniform(1e9, 60e9))
        mb = int(rng.integers(1, 64))
        got = api.plan_batches(vox, t, share, 640.0, mb)
        assert np.array_equal(got, _restated(vox, t, share, 640.0, mb))


def test_rule_cases():
    # capacity: 3 volumes of 1 GB estimate each into a 2.5 GB share
    v = np.full(3, 10 ** 9 // 640, np.int64)
    assert list(api.plan_batches(v, 0.04, int(2.5e9))) == [0, 0, 1]
    # a change of t starts a new batch; max_batch splits
    assert list(api.plan_batches([10, 10, 10, 10], [0.04, 0.04, 0.1, 0.1], 10 ** 9, max_batch=1)) == [0, 1, 2, 3]
    assert list(api.plan_batches([10, 10, 10, 10], [0.04, 0.04, 0.1, 0.1], 10 ** 9)) == [0, 0, 1, 1]
    # a volume alone above the share is refused and does not break the batch around it
    assert list(api.plan_batches([10, 10 ** 9, 10], 0.04, 10 ** 6)) == [0, -1, 0]


def test_rule_argument_errors():
    with pytest.raises(_lib.VoxelCoreError):
        api.plan_batches([1, 2], 0.04, 0)
    with pytest.raises(_lib.VoxelCoreError):
        api.plan_batches([1, 2], 0.04, 100, max_batch=0)
