"""The autotuner (vc_autotune) times the input-dependent launch shapes on the
installed input and keeps the fastest; results never depend on the shapes,
so the tuned path must still reproduce the oracle exactly, for one volume
and for a batch."""
import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import volumes

pytestmark = pytest.mark.gpu


def test_autotune_keeps_results(gpu_ctx):
    ctx = gpu_ctx
    occ = volumes.grf(48, sigma=4.0, seed=3)
    ref = O.run_plain(occ, t=0.04)
    ctx.set_volume(occ)
    tuned = ctx.autotune(0.04)
    assert tuned["ft_ring"] in (4, 8, 16) and tuned["ft_method"] in ("envelope", "window")
    assert tuned["ft_window_ms"] > 0
    assert (tuned["thin_threads"], tuned["thin_blocks_per_sm"], tuned["thin_items"]) in (
        (512, 2, 1), (512, 2, 2), (512, 4, 1), (256, 8, 1), (1024, 1, 1))
    assert all(v > 0 for v in tuned["ft_ms"].values()) and all(v > 0 for v in tuned["thin_ms"].values())
    r = ctx.run_plain(occ, 0.04)
    fl = ctx.thin_flags()
    assert r["thresh"] == ref["thresh"]
    for k in ("keep_v", "keep_e", "keep_f"):
        assert np.array_equal(fl[k], ref["thin"][k]), k
    # every shape gives the same surviving set
    for shape in ((512, 4, 1), (256, 8, 1), (1024, 1, 1), (512, 2, 2), (512, 2, 1)):
        ctx.debug_thin_shape(*shape)
        ctx.run_plain(occ, 0.04)
        fl2 = ctx.thin_flags()
        for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
            assert np.array_equal(fl2[k], ref["thin"][k]), (shape, k)
    ctx.debug_thin_shape(0, 0, 0)
    ctx.set_ft_method("auto")


def test_autotune_on_a_batch(gpu_ctx):
    ctx = gpu_ctx
    vols = [volumes.csg(50 + i, 16, 40) for i in range(5)]
    ctx.batch_set_volumes(vols)
    ctx.autotune(0.04)
    res = ctx.batch_run(0.04)
    for v, r in zip(vols, res):
        ref = O.run_plain(v, t=0.04)
        assert (r["rem"]["nv"], r["rem"]["ne"], r["rem"]["nt"]) == (
            len(ref["rem_vts"]), len(ref["rem_edges"]), len(ref["rem_tris"]))
    ctx.debug_thin_shape(0, 0, 0)
    ctx.set_ft_method("auto")
