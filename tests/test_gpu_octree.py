"""Octree (.sof) volumes on the GPU (vc_set_volume_sof): the decoded
occupancy and the octree sites against the reference's own reading of the
same files (tests/golden/golden_sof.npz), and the feature transform and
lattice complex built on them against the oracle."""
import os

import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import _lib

pytestmark = pytest.mark.gpu
ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture(scope="module")
def sof_golden():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_sof.npz")))


NAMES = ["csg13", "grf32", "noise", "spheres30", "torus40"]


@pytest.mark.parametrize("name", NAMES)
def test_sof_volume_and_sites_match_reference(gpu_ctx, sof_golden, name):
    g = sof_golden
    ctx = gpu_ctx
    n = ctx.set_volume_sof(g[f"sof_{name}"].tobytes())
    assert n == int(g[f"sofsize_{name}"][0])
    occ = ctx.volume()
    assert np.array_equal(np.packbits(occ.ravel()), g[f"sofocc_{name}"])
    ns = ctx.extract_sites()
    ref_sites = g[f"sofsites_{name}"].astype(np.float32) - 0.5
    assert ns == len(ref_sites)
    assert np.array_equal(ctx.sites(), ref_sites)
    # the transform and the lattice complex on the octree's sites
    lat = (ref_sites + 0.5).astype(np.int64)  # lattice points of the sites
    li = (lat[:, 0] * (n + 1) + lat[:, 1]) * (n + 1) + lat[:, 2]
    d2_ref, ids_ref = O.ft(occ.shape, li.astype(np.int64))
    ctx.feature_transform()
    d2, ids = ctx.ft()
    assert np.array_equal(d2, d2_ref) and np.array_equal(ids, ids_ref)
    vd_ref = O.lattice_vd(occ, ids_ref, ref_sites)
    s = ctx.lattice_vd()
    vd = ctx.vd()
    assert (s["nv"], s["ne"], s["nt"]) == (len(vd_ref["vts"]), len(vd_ref["edges"]), len(vd_ref["tris"]))
    for k in ("vts", "edges", "tris", "fm"):
        assert np.array_equal(vd[k], vd_ref[k]), k


def test_malformed_sof_is_rejected(gpu_ctx, sof_golden):
    data = sof_golden["sof_grf32"].tobytes()
    for bad in (data[:-3], np.int32(24).tobytes() + data[4:], b"\x01"):
        with pytest.raises(_lib.VoxelCoreError) as ei:
            gpu_ctx.set_volume_sof(bad)
        assert ei.value.status == _lib.VC_ERR_ARG
    # the context stays usable, and a dense volume afterwards uses the dense site rule
    occ = np.ones((4, 5, 6), np.uint8)
    gpu_ctx.set_volume(occ)
    assert gpu_ctx.extract_sites() == len(O.extract_sites(occ)[0])
