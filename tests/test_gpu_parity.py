"""GPU parity: every stage of the sm_103a library, called through the C ABI,
against the CPU oracle (itself pinned to the reference's compiled sources)
and against the golden vectors recorded from the reference.  Integer and
index results must be bit-identical; lambda measures are exact too (integer
squared distances below 2^24 and a correctly rounded square root)."""
import numpy as np
import pytest

import oracle as O
from complexes import grid_surface, octahedron_shell, random_measures
from helpers import golden_flags, golden_volume, golden_volume_names, lattice_case, rem_hash
from voxel_ma_gb300 import _lib, volumes

pytestmark = pytest.mark.gpu


def _volumes():
    rng = np.random.default_rng(9)
    yield "torus64", volumes.torus_mesh(64)
    yield "grf48", volumes.grf(48, sigma=6.0, seed=1)
    yield "spheres64", volumes.spheres(64, count=32, seed=0)
    yield "csg", volumes.csg(2, 32, 64)
    yield "noise", (rng.uniform(size=(17, 23, 31)) < 0.5).astype(np.uint8)
    yield "tiny", np.ones((1, 1, 1), np.uint8)
    yield "full", np.ones((6, 7, 8), np.uint8)


VOLS = list(_volumes())


@pytest.mark.parametrize("name,occ", VOLS, ids=[v[0] for v in VOLS])
def test_sites_ft_vd_match_oracle(gpu_ctx, name, occ):
    ctx = gpu_ctx
    L = lattice_case(O, occ)
    ctx.set_volume(occ)
    n = ctx.extract_sites()
    assert n == len(L["xyz"])
    assert np.array_equal(ctx.sites(), L["xyz"])
    ctx.feature_transform()
    d2, ids = ctx.ft()
    assert np.array_equal(d2, L["d2"]), "squared distances differ"
    assert np.array_equal(ids, L["ids"]), "nearest-site indices differ"
    s = ctx.lattice_vd()
    vd = ctx.vd()
    ovd = L["vd"]
    assert (s["nv"], s["ne"], s["nt"]) == (len(ovd["vts"]), len(ovd["edges"]), len(ovd["tris"]))
    assert s["inside_size"] == ovd["inside_size"]
    for k in ("vts", "edges", "tris", "vm", "em", "fm", "tri_face", "face_sites"):
        assert np.array_equal(vd[k], ovd[k]), k
    assert np.array_equal(ctx.vertex_radii(), ovd["radius"]), "radius"
    # the lattice complex is installed already finalized: its adjacency must be
    # what cellcomplex::finalize builds from (vts, edges, tris)
    ctx.use_vd_as_complex()
    fin = ctx.finalized()
    for k in ("edges", "tri_edges", "ve_off", "ve_ids", "ef_off", "ef_ids"):
        assert np.array_equal(fin[k], L["fin"][k]), k


def _sparse_volume():
    occ = np.zeros((150, 140, 130), np.uint8)
    occ[10:14, 12:15, 9:13] = 1
    occ[120:125, 100:104, 90:95] = 1
    return occ


FT_VOLS = [VOLS[0], VOLS[2], VOLS[3], VOLS[4],
           ("rod", (np.random.default_rng(3).uniform(size=(2, 300, 3)) < 0.3).astype(np.uint8)),
           ("slab", (np.random.default_rng(4).uniform(size=(260, 2, 5)) < 0.05).astype(np.uint8)),
           # more than 2048 points along z: the 64-bit path is the default there
           ("long", (np.random.default_rng(6).uniform(size=(2, 3, 2100)) < 0.02).astype(np.uint8)),
           # two small blocks in a large box: most lines have points farther
           # than the window kernel scans, and go to the envelope kernel
           ("sparse", _sparse_volume())]


@pytest.mark.parametrize("name,occ", FT_VOLS, ids=[v[0] for v in FT_VOLS])
def test_ft_narrow_and_wide_arithmetic(gpu_ctx, name, occ):
    """Below 2048 points per axis the y and x passes run in 32-bit
    arithmetic, by the envelope kernel or by the window kernel (with the
    envelope kernel for the tiles it leaves); above (or forced) the envelope
    kernel runs in 64-bit.  Every way must give the oracle's exact transform."""
    ctx = gpu_ctx
    L = lattice_case(O, occ)
    try:
        for method, wide in (("envelope", False), ("window", False), ("auto", False), ("envelope", True)):
            ctx.set_ft_method(method)
            ctx.debug_ft_wide(wide)
            ctx.set_volume(occ)
            ctx.extract_sites()
            ctx.feature_transform()
            d2, ids = ctx.ft()
            assert np.array_equal(d2, L["d2"]) and np.array_equal(ids, L["ids"]), (method, wide)
    finally:
        ctx.debug_ft_wide(False)
        ctx.set_ft_method("auto")


def test_empty_volume(gpu_ctx):
    occ = np.zeros((5, 6, 7), np.uint8)
    gpu_ctx.set_volume(occ)
    assert gpu_ctx.extract_sites() == 0
    gpu_ctx.feature_transform()
    d2, ids = gpu_ctx.ft()
    assert (ids == -1).all() and (d2 == np.iinfo(np.int32).max).all()
    s = gpu_ctx.lattice_vd()
    assert s["nv"] == s["ne"] == s["nt"] == 0
    assert len(gpu_ctx.vertex_radii()) == 0


def test_sites_match_reference_golden(gpu_ctx, golden):
    for name in golden_volume_names(golden):
        occ = golden_volume(golden, name)
        gpu_ctx.set_volume(occ)
        gpu_ctx.extract_sites()
        ref = golden[f"sites_{name}"].astype(np.float32) - 0.5
        assert np.array_equal(gpu_ctx.sites(), ref), name


def _gpu_thin(ctx, vts, edges, tris, em_fin, fm, thr):
    ctx.set_complex(vts, edges, tris)
    ne = ctx.finalize()
    assert ne == len(em_fin)
    ctx.set_measures(np.zeros(len(vts), np.float32), em_fin, fm)
    st = ctx.thin(thr, thr)
    return st, ctx.thin_flags()


@pytest.mark.parametrize("seed", range(10))
def test_finalize_and_thin_generic_complexes(gpu_ctx, seed):
    rng = np.random.default_rng(200 + seed)
    vts, edges, tris = grid_surface(int(rng.integers(3, 40)), int(rng.integers(3, 40)), seed=seed,
                                    drop=float(rng.uniform(0, 0.3)), extra_edges=int(rng.integers(0, 40)),
                                    unsorted=float(rng.uniform(0, 0.3)), omit=float(rng.uniform(0, 0.3)))
    fin = O.finalize(len(vts), edges, tris)
    gpu_ctx.set_complex(vts, edges, tris)
    gpu_ctx.finalize()
    g = gpu_ctx.finalized()
    for k in ("edges", "tri_edges", "ve_off", "ve_ids", "ef_off", "ef_ids"):
        assert np.array_equal(g[k], fin[k]), k
    _, em, fm = random_measures(len(fin["edges"]), len(tris), seed=seed, levels=int(rng.integers(2, 6)))
    for thr in (0.5, 1.0, 2.0, 9.0):
        r = O.thin(len(vts), edges, tris, em, fm, thr, thr)
        st, fl = _gpu_thin(gpu_ctx, vts, edges, tris, em, fm, thr)
        for key in ("keep_v", "keep_e", "keep_f", "removed_e"):
            assert np.array_equal(fl[key], r[key]), (thr, key)
        assert st["processed"] == r["stats"]["processed"]


@pytest.mark.parametrize("case", ["grid_a", "grid_b", "grid_c", "octa"])
@pytest.mark.parametrize("tag", ["lo", "hi"])
def test_thin_matches_reference_golden(gpu_ctx, golden, case, tag):
    vts, edges, tris, em, fm = (golden[f"cc_{case}_{k}"] for k in ("vts", "edges", "tris", "em", "fm"))
    p = f"cc_{case}_{tag}_"
    thr = float(golden[p + "thr"][0])
    st, fl = _gpu_thin(gpu_ctx, vts, edges, tris, em, fm, thr)
    g = gpu_ctx.finalized()
    assert np.array_equal(g["edges"], golden[f"cc_{case}_fin_edges"])
    assert np.array_equal(g["tri_edges"], golden[f"cc_{case}_fin_tri_edges"])
    for k, n in (("keep_v", len(vts)), ("keep_e", len(em)), ("keep_f", len(tris)), ("removed_e", len(em))):
        assert np.array_equal(fl[k], golden_flags(golden, p + k, n)), k
    gpu_ctx.remaining()
    rv, re_, rt = gpu_ctx.remaining_arrays()
    assert [len(rv), len(re_), len(rt)] == list(golden[p + "rem_sizes"])
    assert rem_hash(rv, re_, rt) == golden[p + "rem_hash"].tobytes()
    eu = gpu_ctx.euler_remaining()
    assert [eu["V"], eu["E"], eu["F"], eu["C"], eu["euler"]] == list(golden[p + "euler"])


@pytest.mark.parametrize("name", ["torus32", "grf24", "spheres28", "csg11", "edge_touch"])
def test_lattice_pipeline_matches_reference_golden(gpu_ctx, golden, name):
    occ = golden_volume(golden, name)
    for t in (0.04, 0.2):
        p = f"vd_{name}_{t}_"
        r = gpu_ctx.run_plain(occ, t)
        assert r["thresh"] == float(golden[p + "thr"][0])
        sizes = golden[f"vd_{name}_sizes"]
        assert [r["vd"]["nv"], r["vd"]["ne"], r["vd"]["nt"]] == list(sizes)
        fl = gpu_ctx.thin_flags()
        for k, n in (("keep_v", sizes[0]), ("keep_e", sizes[1]), ("keep_f", sizes[2])):
            assert np.array_equal(fl[k], golden_flags(golden, p + k, int(n))), (t, k)
        assert [r["rem"]["nv"], r["rem"]["ne"], r["rem"]["nt"]] == list(golden[p + "rem_sizes"])
        eu = gpu_ctx.euler_remaining()
        assert [eu["V"], eu["E"], eu["F"], eu["C"], eu["euler"]] == list(golden[p + "euler"])


@pytest.mark.parametrize("name,occ", VOLS[:4], ids=[v[0] for v in VOLS[:4]])
@pytest.mark.parametrize("t", [0.0, 0.04, 0.1])
def test_plain_path_matches_oracle(gpu_ctx, name, occ, t):
    ref = O.run_plain(occ, t=t)
    r = gpu_ctx.run_plain(occ, t)
    assert r["thresh"] == ref["thresh"]
    fl = gpu_ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
        assert np.array_equal(fl[k], ref["thin"][k]), k
    assert r["thin"]["processed"] == ref["thin"]["stats"]["processed"]
    rv, re_, rt = gpu_ctx.remaining_arrays()
    assert np.array_equal(rv, ref["rem_vts"]) and np.array_equal(re_, ref["rem_edges"])
    assert np.array_equal(rt, ref["rem_tris"])
    eu = gpu_ctx.euler_remaining()
    assert eu == O.euler(len(rv), re_, rt)


def _boundary_shapes():
    # lattice rows of 32, 33, 64 and 96 points (segment and word edges), odd
    # and one-voxel extents
    rng = np.random.default_rng(21)
    for shape in [(6, 5, 31), (4, 7, 32), (5, 3, 63), (3, 4, 95), (9, 1, 40), (1, 9, 33), (40, 6, 1)]:
        yield f"box{shape}", volumes.grf(max(shape), sigma=2.5, seed=sum(shape))[: shape[0], : shape[1], : shape[2]]
        yield f"noise{shape}", (rng.uniform(size=shape) < 0.6).astype(np.uint8)


BOUNDARY = list(_boundary_shapes())


@pytest.mark.parametrize("name,occ", BOUNDARY, ids=[v[0] for v in BOUNDARY])
def test_plain_path_at_segment_boundaries(gpu_ctx, name, occ):
    """Rows whose lengths sit on the 32-point segment and 32-voxel word edges:
    every stage of the plain path equals the oracle."""
    occ = np.ascontiguousarray(occ)
    ref = O.run_plain(occ, t=0.04)
    r = gpu_ctx.run_plain(occ, 0.04)
    assert r["n_sites"] == len(ref["sites"])
    assert np.array_equal(gpu_ctx.sites(), ref["sites"])
    d2, ids = gpu_ctx.ft()
    assert np.array_equal(d2, ref["d2"]) and np.array_equal(ids, ref["ids"])
    vd = gpu_ctx.vd()
    for k in ("vts", "edges", "tris", "vm", "em", "fm", "tri_face", "face_sites"):
        assert np.array_equal(vd[k], ref["vd"][k]), k
    fl = gpu_ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
        assert np.array_equal(fl[k], ref["thin"][k]), k
    rv, re_, rt = gpu_ctx.remaining_arrays()
    assert np.array_equal(rv, ref["rem_vts"]) and np.array_equal(re_, ref["rem_edges"])
    assert np.array_equal(rt, ref["rem_tris"])


def test_closed_pocket_and_errors(gpu_ctx):
    vts, edges, tris = octahedron_shell()
    st, fl = _gpu_thin(gpu_ctx, vts, edges, tris, np.zeros(12, np.float32), np.zeros(8, np.float32), 1.0)
    assert fl["keep_f"].all() and st["processed"] == 0
    # a triangle with a repeated vertex is rejected, not thinned
    bad = np.array([[0, 0, 1]], np.int32)
    gpu_ctx.set_complex(vts, np.zeros((0, 2), np.int32), bad)
    with pytest.raises(_lib.VoxelCoreError) as ei:
        gpu_ctx.finalize()
    assert ei.value.status == _lib.VC_ERR_ARG
    # the context stays usable after the rejected call
    st, fl = _gpu_thin(gpu_ctx, vts, edges, tris, np.zeros(12, np.float32), np.zeros(8, np.float32), 1.0)
    assert fl["keep_f"].all()


def test_call_order_is_checked(gpu_ctx):
    from voxel_ma_gb300 import api
    ctx = api.Context(0)
    try:
        with pytest.raises(_lib.VoxelCoreError) as ei:
            ctx.feature_transform()
        assert ei.value.status == _lib.VC_ERR_STATE
    finally:
        ctx.close()


def test_device_resident_inputs(gpu_ctx):
    torch = pytest.importorskip("torch")
    occ = volumes.torus_mesh(32)
    ref = O.run_plain(occ, t=0.04)
    r = gpu_ctx.run_plain(torch.from_numpy(occ).cuda(), 0.04)
    fl = gpu_ctx.thin_flags(device=True)
    assert np.array_equal(fl["keep_f"].cpu().numpy(), ref["thin"]["keep_f"])
    assert r["rem"]["nt"] == len(ref["rem_tris"])


def test_lambda_fp64_check(gpu_ctx):
    """Face lambdas are correctly rounded square roots of exact integers, so
    against an FP64 recomputation their relative error is at most 2^-24; the
    threshold-flip count is reported (the path keeps float semantics)."""
    occ = volumes.grf(40, sigma=3.0, seed=11)
    gpu_ctx.run_plain(occ, 0.04)
    chk = gpu_ctx.lambda_fp64_check()
    assert 0.0 <= chk["max_rel_err"] <= 2.0 ** -24
    assert chk["flips"] >= 0
    gpu_ctx.set_volume(occ)
    gpu_ctx.extract_sites()
    gpu_ctx.feature_transform()
    gpu_ctx.lattice_vd()  # no thresholds: flips not counted
    assert gpu_ctx.lambda_fp64_check()["flips"] == -1



def _closed_cases():
    yield "octahedron", octahedron_shell()
    for seed in range(3):
        rng = np.random.default_rng(100 + seed)
        yield f"grid{seed}", grid_surface(int(rng.integers(3, 30)), int(rng.integers(3, 30)), seed=seed)


@pytest.mark.parametrize("name,cx", list(_closed_cases()), ids=[c[0] for c in _closed_cases()])
def test_closed_components_generic(gpu_ctx, name, cx):
    vts, edges, tris = cx
    gpu_ctx.set_complex(vts, edges, tris)
    gpu_ctx.finalize()
    assert gpu_ctx.closed_components() == O.closed_components(len(vts), edges, tris)


@pytest.mark.parametrize("name,occ", VOLS[:4], ids=[v[0] for v in VOLS[:4]])
def test_closed_components_lattice(gpu_ctx, name, occ):
    """nClosedComponents of the lattice complex: the pockets of the discrete
    Voronoi regions; also the all-pass thinning's flags against the oracle."""
    ctx = gpu_ctx
    L = lattice_case(O, occ)
    vd = L["vd"]
    ctx.set_volume(occ)
    ctx.extract_sites()
    ctx.feature_transform()
    ctx.lattice_vd()
    ctx.use_vd_as_complex()
    n = ctx.closed_components()
    assert n == O.closed_components(len(vd["vts"]), vd["edges"], vd["tris"])
    ref = O.thin(len(vd["vts"]), vd["edges"], vd["tris"], np.zeros(len(L["em_fin"]), np.float32),
                 np.zeros(len(vd["tris"]), np.float32), 1.0, 1.0)
    fl = ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
        assert np.array_equal(fl[k], ref[k]), k
    # the thinning with the lattice complex's own measures is unaffected
    thr = float(np.float32(np.float64(vd["inside_size"]) * 0.04))
    st = ctx.thin(thr, thr)
    r = O.thin(len(vd["vts"]), vd["edges"], vd["tris"], L["em_fin"], vd["fm"], thr, thr)
    fl = ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f"):
        assert np.array_equal(fl[k], r[k]), k


def test_remaining_is_idempotent(gpu_ctx):
    """vc_remaining called again after the same thinning returns the same
    complex (the reference's remainingCC can be called any number of times)."""
    ctx = gpu_ctx
    vts, edges, tris = grid_surface(12, 9, seed=3, drop=0.2, extra_edges=8)
    fin = O.finalize(len(vts), edges, tris)
    _, em, fm = random_measures(len(fin["edges"]), len(tris), seed=3, levels=3)
    ctx.set_complex(vts, edges, tris)
    ctx.finalize()
    ctx.set_measures(np.zeros(len(vts), np.float32), em, fm)
    ctx.thin(1.0, 1.0)
    first = (ctx.remaining(), *ctx.remaining_arrays())
    for _ in range(2):
        again = (ctx.remaining(), *ctx.remaining_arrays())
        assert again[0] == first[0]
        for a, b in zip(again[1:], first[1:]):
            assert np.array_equal(a, b)
    r = O.thin(len(vts), edges, tris, em, fm, 1.0, 1.0)
    rv, re_, rt = O.remaining(vts, fin["edges"], tris, r["keep_v"], r["keep_e"], r["keep_f"])
    assert np.array_equal(first[1], rv) and np.array_equal(first[2], re_) and np.array_equal(first[3], rt)
