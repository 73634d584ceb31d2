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


def test_uniform_cube_has_no_sites(gpu_ctx):
    # the whole cube one empty node: no subtree for the walker, no sites
    for sign, inside in ((1, 0), (0, 1), (2, 1)):
        data = np.int32(64).tobytes() + bytes([1, sign])
        assert gpu_ctx.set_volume_sof(data) == 65
        assert np.array_equal(gpu_ctx.volume(), np.full((65, 65, 65), inside, np.uint8))
        assert gpu_ctx.extract_sites() == 0


def test_malformed_subtree_is_rejected_on_the_device(gpu_ctx, sof_golden):
    bad = [
        np.int32(32).tobytes() + bytes([0]) + bytes([2, 0x0F]) * 8,    # a leaf of 16^3 cells
        np.int32(2).tobytes() + bytes([0, 0]) + bytes([1, 1]) * 15,    # an internal node of one cell
    ]
    for data in bad:
        assert O.sof_decode(data) is None
        with pytest.raises(_lib.VoxelCoreError) as ei:
            gpu_ctx.set_volume_sof(data)
        assert ei.value.status == _lib.VC_ERR_ARG
    # the context stays usable
    g = sof_golden
    n = gpu_ctx.set_volume_sof(g["sof_grf32"].tobytes())
    assert np.array_equal(np.packbits(gpu_ctx.volume().ravel()), g["sofocc_grf32"])
    assert n == int(g["sofsize_grf32"][0])


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_encoded_volumes_decode_like_the_oracle(gpu_ctx, seed):
    # sizes past 16 per axis: empty nodes above the walker's subtrees, and
    # subtrees of every depth
    from voxel_ma_gb300 import api, volumes
    rng = np.random.default_rng(seed)
    shape = tuple(int(v) for v in rng.integers(20, 140, size=3))
    occ = volumes.csg(100 + seed, 20, 140)
    occ = occ[: shape[0], : shape[1], : shape[2]]
    data = api.encode_sof(occ)
    occ_ref, sites_ref = O.sof_decode(data)
    n = gpu_ctx.set_volume_sof(data)
    assert (n, n, n) == occ_ref.shape
    assert np.array_equal(gpu_ctx.volume(), occ_ref)
    assert np.array_equal(gpu_ctx.volume()[: occ.shape[0], : occ.shape[1], : occ.shape[2]], occ > 0)
    assert gpu_ctx.extract_sites() == len(sites_ref)
    assert np.array_equal(gpu_ctx.sites(), np.asarray(sites_ref, np.float32))


@pytest.mark.parametrize("name", NAMES)
def test_sog_volume_and_sites_match_reference(gpu_ctx, sof_golden, name):
    g = sof_golden
    n = gpu_ctx.set_volume_sog(g[f"sog_{name}"].tobytes())
    assert n == int(g[f"sofsize_{name}"][0])
    assert np.array_equal(np.packbits(gpu_ctx.volume().ravel()), g[f"sogocc_{name}"])
    assert gpu_ctx.extract_sites() == len(g[f"sogsites_{name}"])
    assert np.array_equal(gpu_ctx.sites(), g[f"sogsites_{name}"].astype(np.float32) - 0.5)
    assert np.array_equal(gpu_ctx.vox_to_model(), np.eye(4))  # lower-left 0, length R


def _run_installed(ctx, t=0.04):
    ctx.extract_sites()
    ctx.feature_transform()
    s = ctx.lattice_vd()
    thr = float(np.float32(np.float64(s["inside_size"]) * t))
    ctx.thin(thr, thr)
    ctx.remaining()


def test_sog_transform_reaches_the_written_files(gpu_ctx, sof_golden, tmp_path):
    """A .sog header with lower-left (1.5, -2, 3.25) and length 2R: the
    written vertices are 2v + lower-left (one double expression rounded to
    float, as trimesh's xform * point), the radii len(M (r,0,0) - M 0)."""
    ctx = gpu_ctx
    base = sof_golden["sog_torus40"].tobytes()
    R = int(np.frombuffer(base[128:132], np.int32)[0])
    ll = np.array([1.5, -2.0, 3.25], np.float32)
    moved = base[:15] + ll.tobytes() + np.float32(2 * R).tobytes() + base[31:]
    ctx.set_volume_sog(base)
    _run_installed(ctx)
    ctx.write_remaining(str(tmp_path / "id"))
    v, e, t = ctx.remaining_arrays()
    keep = ctx.thin_flags()["keep_v"].astype(bool)
    r = ctx.vertex_radii()[keep]
    O.write_ply(str(tmp_path / "o_id.ply"), v, e, t)
    assert open(str(tmp_path / "id.ply"), "rb").read() == open(str(tmp_path / "o_id.ply"), "rb").read()
    ctx.set_volume_sog(moved)
    M = ctx.vox_to_model()
    assert np.array_equal(M, np.array([[2, 0, 0, 1.5], [0, 2, 0, -2], [0, 0, 2, 3.25], [0, 0, 0, 1]], np.float64))
    _run_installed(ctx)
    ctx.write_remaining(str(tmp_path / "mv"))
    tv = (2.0 * v.astype(np.float64) + ll.astype(np.float64)).astype(np.float32)
    q = (2.0 * r.astype(np.float64) + np.float64(ll[0])).astype(np.float32)
    d = (q - ll[0]).astype(np.float32)
    rr = np.sqrt(d * d).astype(np.float32)
    O.write_ply(str(tmp_path / "o.ply"), tv, e, t)
    O.write_radii(str(tmp_path / "o.r"), tv, rr)
    O.write_dotma(str(tmp_path / "o.ma"), tv, rr, O.dotma_edges(e, t), t)
    for ext in (".ply", ".r", ".ma"):
        assert open(str(tmp_path / "mv") + ext, "rb").read() == open(str(tmp_path / "o") + ext, "rb").read(), ext


def test_malformed_sog_is_rejected(gpu_ctx, sof_golden):
    data = sof_golden["sog_grf32"].tobytes()
    for bad in (data[:-5], b"SOG.Format 2.0\0" + data[15:], data[:100]):
        with pytest.raises(_lib.VoxelCoreError) as ei:
            gpu_ctx.set_volume_sog(bad)
        assert ei.value.status == _lib.VC_ERR_ARG
