"""The batched path (vc_batch_set_volumes + vc_batch_run): one pass of the
pipeline over volumes of uneven sizes must give every volume exactly what the
plain single-volume path gives for it alone -- sites, surviving cell set,
threshold, remaining complex and its Euler characteristic -- and what the
oracle gives."""
import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import _lib, api, volumes

pytestmark = pytest.mark.gpu


def _batch(seed=3):
    rng = np.random.default_rng(seed)
    vols = [volumes.csg(100 + i, 12, 40) for i in range(8)]
    vols.append((rng.uniform(size=(9, 17, 5)) < 0.5).astype(np.uint8))
    vols.append(np.zeros((6, 5, 4), np.uint8))           # no sites, no cells
    vols.append(np.ones((1, 1, 1), np.uint8))            # one voxel
    vols.append(volumes.spheres(24, count=4, seed=5))
    vols.append(np.ones((7, 3, 9), np.uint8))            # full box
    vols.append(volumes.torus_mesh(32))
    return vols


@pytest.fixture(scope="module")
def plain_ctx(gpu_ctx):
    c = api.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("t,method", [(0.04, "envelope"), (0.2, "envelope"), (0.04, "window")])
def test_batch_equals_each_volume_alone(gpu_ctx, plain_ctx, t, method):
    """(The window method's tiles span several of these small volumes.)"""
    vols = _batch()
    gpu_ctx.set_ft_method(method)
    gpu_ctx.batch_set_volumes(vols)
    try:
        res = gpu_ctx.batch_run(t=t, euler=True)
    finally:
        gpu_ctx.set_ft_method("auto")
    parts = gpu_ctx.batch_split(res)
    assert len(res) == len(vols)
    for i, (occ, r, part) in enumerate(zip(vols, res, parts)):
        p = plain_ctx.run_plain(occ, t=t)
        assert r["n_sites"] == p["n_sites"], i
        assert np.array_equal(part["sites"], plain_ctx.sites()), i
        assert r["vd"] == p["vd"], i
        assert np.float32(r["thresh"]) == np.float32(p["thresh"]), i
        fl = plain_ctx.thin_flags()
        for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
            assert np.array_equal(part[k], fl[k]), (i, k)
        assert r["rem"] == p["rem"], i
        rv, re_, rt = plain_ctx.remaining_arrays()
        assert np.array_equal(part["rem_vts"], rv), i
        assert np.array_equal(part["rem_edges"], re_), i
        assert np.array_equal(part["rem_tris"], rt), i
        eu = plain_ctx.euler_remaining()
        assert r["euler"] == eu, i


def test_batch_matches_oracle(gpu_ctx):
    vols = _batch(seed=4)[:6]
    gpu_ctx.batch_set_volumes(vols)
    res = gpu_ctx.batch_run(t=0.04, euler=True)
    parts = gpu_ctx.batch_split(res)
    for occ, r, part in zip(vols, res, parts):
        ref = O.run_plain(occ, t=0.04)
        assert np.array_equal(part["sites"], ref["sites"])
        assert np.float32(r["thresh"]) == np.float32(ref["thresh"])
        for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
            assert np.array_equal(part[k], ref["thin"][k]), k
        assert np.array_equal(part["rem_vts"], ref["rem_vts"])
        assert np.array_equal(part["rem_edges"], ref["rem_edges"])
        assert np.array_equal(part["rem_tris"], ref["rem_tris"])
        assert r["euler"] == O.euler(len(ref["rem_vts"]), ref["rem_edges"], ref["rem_tris"])


def test_batch_of_one_and_device_input(gpu_ctx, plain_ctx):
    torch = pytest.importorskip("torch")
    occ = volumes.csg(9, 20, 36)
    gpu_ctx.batch_set_volumes([torch.from_numpy(occ).cuda()])
    r = gpu_ctx.batch_run(t=0.04)[0]
    p = plain_ctx.run_plain(occ, t=0.04)
    assert r["rem"] == p["rem"] and r["vd"] == p["vd"]
    # the same context then runs the plain path: records are rebuilt from the measures
    q = gpu_ctx.run_plain(occ, t=0.04)
    assert q["rem"] == p["rem"]
    assert np.array_equal(gpu_ctx.thin_flags()["keep_e"], plain_ctx.thin_flags()["keep_e"])


def test_batch_argument_errors(gpu_ctx):
    import ctypes
    occ = np.ones(8, np.uint8)
    dims = np.array([[2, 2, 2], [0, 1, 1]], np.int32)
    s = gpu_ctx.lib.vc_batch_set_volumes(gpu_ctx.h, 2, dims.ctypes.data_as(ctypes.c_void_p),
                                          occ.ctypes.data_as(ctypes.c_void_p), _lib.VC_MEM_HOST)
    assert s == _lib.VC_ERR_ARG
    s = gpu_ctx.lib.vc_batch_set_volumes(gpu_ctx.h, 0, dims.ctypes.data_as(ctypes.c_void_p),
                                          occ.ctypes.data_as(ctypes.c_void_p), _lib.VC_MEM_HOST)
    assert s == _lib.VC_ERR_ARG
