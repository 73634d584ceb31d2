"""The thinning queue's positions and capacity, on small complexes.

Queue positions are unsigned 32-bit and a cell's last-decrement record holds
(position << 1 | slot) in 64 bits: on the 1024^3 random field (V + E = 2.6e9
cells, about 2.2e9 pushes) positions pass 2^31.  The queue holds V + E + 1
items per generation when that fits in device memory and otherwise what is
free; a generation beyond the capacity ends the thinning with VC_ERR_OOM.
Both are exercised here without a large complex: the first position is moved
up (so that every position lies above 2^31, or the positions cross it), and
the capacity is set to the largest generation (the same flags and remaining
complex as the oracle's) and to one item less (VC_ERR_OOM, and the context
then thins exactly again)."""
import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import _lib, volumes

pytestmark = pytest.mark.gpu


def _same_as_oracle(ctx, ref):
    fl = ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
        assert np.array_equal(fl[k], ref["thin"][k]), k
    rv, re_, rt = ctx.remaining_arrays()
    assert np.array_equal(rv, ref["rem_vts"]) and np.array_equal(re_, ref["rem_edges"])
    assert np.array_equal(rt, ref["rem_tris"])


@pytest.fixture(scope="module")
def case():
    occ = volumes.grf(48, sigma=3.0, seed=7)
    return occ, O.run_plain(occ, 0.04)


def _largest_generation(ctx, occ):
    ctx.debug_thin_trace(4096)
    try:
        r = ctx.run_plain(occ, 0.04)
        tr = ctx.thin_trace()
    finally:
        ctx.debug_thin_trace(0)
    assert len(tr) == r["thin"]["generations"]
    return r, int(tr[:, 0].max())


def test_positions_above_2_31(gpu_ctx, case):
    occ, ref = case
    ctx = gpu_ctx
    r, _ = _largest_generation(ctx, occ)
    ncell = r["vd"]["nv"] + r["vd"]["ne"]
    try:
        for first in (2**31 - 5, 2**31 + 12345, 2**32 - ncell - 9):
            ctx.debug_thin_queue(0, first)
            r2 = ctx.run_plain(occ, 0.04)
            assert r2["thin"] == r["thin"], first
            assert r2["thin"]["processed"] == ref["thin"]["stats"]["processed"]
            _same_as_oracle(ctx, ref)
        # the generic path (records built from the complex and its measures)
        ctx.debug_thin_queue(0, 2**32 - ncell - 9)
        ctx.thin(ref["thresh"], ref["thresh"])
        ctx.remaining()
        _same_as_oracle(ctx, ref)
        # positions past 2^32 - 1 cannot be represented
        ctx.debug_thin_queue(0, 2**32 - ncell - 1)
        with pytest.raises(_lib.VoxelCoreError) as ei:
            ctx.run_plain(occ, 0.04)
        assert ei.value.status == _lib.VC_ERR_ARG
    finally:
        ctx.debug_thin_queue(0, 0)
    ctx.run_plain(occ, 0.04)
    _same_as_oracle(ctx, ref)


def test_capacity_of_the_largest_generation(gpu_ctx, case):
    occ, ref = case
    ctx = gpu_ctx
    r, m = _largest_generation(ctx, occ)
    assert 0 < m < r["vd"]["nv"] + r["vd"]["ne"]
    try:
        ctx.debug_thin_queue(m, 2**31 - 77)
        r2 = ctx.run_plain(occ, 0.04)
        assert r2["thin"] == r["thin"]
        _same_as_oracle(ctx, ref)
        ctx.debug_thin_queue(m - 1, 0)
        with pytest.raises(_lib.VoxelCoreError) as ei:
            ctx.run_plain(occ, 0.04)
        assert ei.value.status == _lib.VC_ERR_OOM
    finally:
        ctx.debug_thin_queue(0, 0)
    r3 = ctx.run_plain(occ, 0.04)
    assert r3["thin"] == r["thin"]
    _same_as_oracle(ctx, ref)
