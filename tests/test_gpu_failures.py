"""Failure paths of the library on the GPU, each made on the host side: no
kernel is made to fault, trap or wait without a limit.

  * a grid barrier of the thinning kernel that gives up (its poll limit set to
    one poll) -> VC_ERR_TIMEOUT, and the same context then thins correctly;
  * a device allocation that fails (the k-th one of a call) -> VC_ERR_OOM at
    every stage of the plain path, in a context and in one request of the
    request loop, and both stay usable;
  * a broken reference count -> VC_ERR_INVARIANT, where the reference's
    logic check (src/ccthin.cpp:570-584) prints and calls exit(1)."""
import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import _lib, api, volumes

pytestmark = pytest.mark.gpu


def _same_as_oracle(ctx, occ, ref):
    fl = ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
        assert np.array_equal(fl[k], ref["thin"][k]), k
    rv, re_, rt = ctx.remaining_arrays()
    assert np.array_equal(rv, ref["rem_vts"]) and np.array_equal(re_, ref["rem_edges"])
    assert np.array_equal(rt, ref["rem_tris"])


@pytest.fixture(scope="module")
def case():
    occ = volumes.grf(40, sigma=3.0, seed=4)
    return occ, O.run_plain(occ, 0.04)


def test_barrier_timeout_then_recovery(gpu_ctx, case):
    occ, ref = case
    ctx = gpu_ctx
    try:
        ctx.debug_set_spin_limit(1)
        with pytest.raises(_lib.VoxelCoreError) as ei:
            ctx.run_plain(occ, 0.04)
        assert ei.value.status == _lib.VC_ERR_TIMEOUT
    finally:
        ctx.debug_set_spin_limit(0)
    r = ctx.run_plain(occ, 0.04)
    assert r["thin"]["processed"] == ref["thin"]["stats"]["processed"]
    _same_as_oracle(ctx, occ, ref)


def test_allocation_failure_at_every_stage(case):
    """A fresh context allocates as it goes; failing its k-th allocation for
    k = 0, 1, 2, ... hits every stage of the plain path in turn.  Each call
    fails with VC_ERR_OOM and the next call on the same context is exact."""
    occ, ref = case
    seen_ok = False
    for k in range(0, 64, 3):
        with api.Context(0) as ctx:
            ctx.debug_fail_alloc_after(k)
            try:
                ctx.run_plain(occ, 0.04)
                seen_ok = True  # the context needed fewer than k + 1 allocations
            except _lib.VoxelCoreError as exc:
                assert exc.status == _lib.VC_ERR_OOM, exc
            ctx.debug_fail_alloc_after(-1)
            ctx.run_plain(occ, 0.04)
            _same_as_oracle(ctx, occ, ref)
        if seen_ok:
            break
    assert seen_ok


def test_allocation_failure_in_one_request(case):
    occ, ref = case
    srv = api.Server(0, workers=1, mem_cap_bytes=8 << 30, max_batch=4)
    try:
        srv.debug_fail_alloc_after(2)
        bad = srv.submit(occ, 0.04)
        rb = srv.wait(bad)
        assert rb["status"] == _lib.VC_ERR_OOM
        srv.release(bad)
        good = srv.submit(occ, 0.04)
        rg = srv.wait(good)
        assert rg["status"] == _lib.VC_OK
        v, e, t = srv.remaining(good, rg)
        assert np.array_equal(v, ref["rem_vts"]) and np.array_equal(e, ref["rem_edges"])
        assert np.array_equal(t, ref["rem_tris"])
        srv.release(good)
        st = srv.stats()
        assert st["failed"] == 1 and st["completed"] == 2
    finally:
        srv.close()


def test_broken_reference_count_is_an_invariant_error(gpu_ctx):
    """A chain of three edges: vertex 0 starts an edge-vertex pair; with its
    count raised after its record is built, popping that pair meets a count
    of 2 instead of 1."""
    ctx = gpu_ctx
    vts = np.zeros((4, 3), np.float32)
    edges = np.array([[0, 1], [1, 2], [2, 3]], np.int32)
    tris = np.zeros((0, 3), np.int32)
    ref = O.thin(4, edges, tris, np.zeros(3, np.float32), np.zeros(0, np.float32), 1.0, 1.0)
    ctx.set_complex(vts, edges, tris)
    ctx.finalize()
    ctx.set_measures(np.zeros(4, np.float32), np.zeros(3, np.float32), np.zeros(0, np.float32))
    try:
        ctx.debug_ref_bias(0, 1)
        with pytest.raises(_lib.VoxelCoreError) as ei:
            ctx.thin(1.0, 1.0)
        assert ei.value.status == _lib.VC_ERR_INVARIANT
    finally:
        ctx.debug_ref_bias(-1, 0)
    ctx.thin(1.0, 1.0)
    fl = ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
        assert np.array_equal(fl[k], ref[k]), k
