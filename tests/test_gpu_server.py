"""The request loop (vc_server_*): volumes submitted while others are on the
GPU are batched with them, and every result -- alone or in the mix -- equals
the plain single-volume result for that volume."""
import time

import numpy as np
import pytest

from voxel_ma_gb300 import _lib, api, volumes

pytestmark = pytest.mark.gpu


def _volumes():
    rng = np.random.default_rng(11)
    vols = [volumes.csg(300 + i, 10, 44) for i in range(10)]
    vols += [volumes.spheres(28, count=6, seed=3), volumes.torus_mesh(24),
             (rng.uniform(size=(13, 7, 19)) < 0.45).astype(np.uint8), np.zeros((4, 4, 4), np.uint8)]
    return vols


def _expect(ctx, occ, t):
    p = ctx.run_plain(occ, t)
    return p, ctx.remaining_arrays(), ctx.euler_remaining()


def _check(srv, rid, res, exp):
    p, (rv, re_, rt), eu = exp
    assert res["status"] == _lib.VC_OK
    assert res["n_sites"] == p["n_sites"] and res["vd"] == p["vd"] and res["rem"] == p["rem"]
    assert np.float32(res["thresh"]) == np.float32(p["thresh"])
    assert res["euler"] == eu
    v, e, t = srv.remaining(rid, res)
    assert np.array_equal(v, rv) and np.array_equal(e, re_) and np.array_equal(t, rt)


def test_results_alone_and_in_the_mix(gpu_ctx):
    vols = _volumes()
    exp = [_expect(gpu_ctx, v, 0.04) for v in vols]
    srv = api.Server(0, workers=2, mem_cap_bytes=4 << 30, max_batch=5)
    try:
        # alone: one request on an idle server
        rid = srv.submit(vols[0], 0.04)
        res = srv.wait(rid, 120.0)
        assert res["batch_size"] == 1
        _check(srv, rid, res, exp[0])
        srv.release(rid)
        # in the mix: a burst, then more requests while the burst is served
        ids = [srv.submit(v, 0.04) for v in vols[:8]]
        time.sleep(0.01)
        ids += [srv.submit(v, 0.04) for v in vols[8:]]
        got = [srv.wait(i, 300.0) for i in ids]
        assert max(r["batch_size"] for r in got) > 1
        for i, r, x in zip(ids, got, exp):
            _check(srv, i, r, x)
            srv.release(i)
        st = srv.stats()
        assert st["completed"] == len(vols) + 1 and st["failed"] == 0 and st["pending"] == 0
    finally:
        srv.close()


def test_mixed_thresholds_and_refusal(gpu_ctx):
    vols = _volumes()[:6]
    ts = [0.04, 0.2, 0.04, 0.04, 0.2, 0.1]
    exp = [_expect(gpu_ctx, v, t) for v, t in zip(vols, ts)]
    srv = api.Server(0, workers=1, mem_cap_bytes=1 << 30, max_batch=8, bytes_per_voxel=640.0)
    try:
        ids = [srv.submit(v, t) for v, t in zip(vols, ts)]
        for i, x in zip(ids, exp):
            _check(srv, i, srv.wait(i, 300.0), x)
        # a volume whose estimate exceeds the share is refused at submission
        with pytest.raises(_lib.VoxelCoreError):
            srv.submit(np.zeros((128, 128, 128), np.uint8), 0.04)
        assert srv.stats()["refused"] == 1
        with pytest.raises(_lib.VoxelCoreError):
            srv.wait(10 ** 9, 1.0)
    finally:
        srv.close()
