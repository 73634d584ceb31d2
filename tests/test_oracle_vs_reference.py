"""Pin the oracle restatement against the reference's OWN compiled sources on
fresh seeded inputs (needs the reference tree; skipped where it is absent)."""
import numpy as np
import pytest

import oracle as O
from complexes import grid_surface, octahedron_shell, random_measures
from helpers import lattice_case
from voxel_ma_gb300 import volumes

pytestmark = pytest.mark.skipif(not O.ref_available() and not O.reference_tree_present(),
                                reason="reference tree not present on this host")


@pytest.fixture(scope="module", autouse=True)
def _built(oracle_lib):
    if not O.ref_available():
        pytest.skip("reference library could not be built")


@pytest.mark.parametrize("seed", range(6))
def test_sites_random_volumes(seed):
    rng = np.random.default_rng(seed)
    shape = tuple(int(x) for x in rng.integers(3, 14, 3))
    occ = (rng.uniform(size=shape) < rng.uniform(0.2, 0.8)).astype(np.uint8)
    xyz, _ = O.extract_sites(occ)
    assert np.array_equal(xyz, O.ref_extract_sites(occ))


def test_sites_edge_cases():
    for occ in (np.zeros((4, 5, 6), np.uint8), np.ones((4, 5, 6), np.uint8), np.ones((1, 1, 1), np.uint8),
                np.eye(5, dtype=np.uint8)[:, :, None].repeat(3, 2)):
        xyz, _ = O.extract_sites(occ)
        assert np.array_equal(xyz, O.ref_extract_sites(occ))


@pytest.mark.parametrize("seed", range(8))
def test_finalize_and_thin_random_complexes(seed):
    rng = np.random.default_rng(100 + seed)
    vts, edges, tris = grid_surface(int(rng.integers(3, 15)), int(rng.integers(3, 15)), seed=seed,
                                    drop=float(rng.uniform(0, 0.3)), extra_edges=int(rng.integers(0, 20)),
                                    unsorted=float(rng.uniform(0, 0.3)), omit=float(rng.uniform(0, 0.3)))
    rc = O.RefComplex(vts, edges, tris)
    fin = O.finalize(len(vts), edges, tris)
    assert np.array_equal(rc.edges(), fin["edges"])
    assert np.array_equal(rc.tri_edges(), fin["tri_edges"])
    for w, k in ((0, "ve"), (1, "ef")):
        offs, ids = rc.adjacency(w)
        assert np.array_equal(offs, fin[k + "_off"]) and np.array_equal(ids, fin[k + "_ids"])
    _, em, fm = random_measures(rc.ne, len(tris), seed=seed, levels=int(rng.integers(2, 6)))
    for thr in (0.5, 1.0, 2.0, 9.0):
        r = O.thin(len(vts), edges, tris, em, fm, thr, thr)
        ref = rc.thin(np.zeros(len(vts), np.float32), em, fm, thr, thr)
        for key in ("keep_v", "keep_e", "keep_f", "removed_e"):
            assert np.array_equal(r[key], ref[key]), (thr, key)
        rv, re_, rt = O.remaining(vts, fin["edges"], tris, r["keep_v"], r["keep_e"], r["keep_f"])
        a, b, c = rc.remaining()
        assert np.array_equal(rv, a) and np.array_equal(re_, b) and np.array_equal(rt, c)
        assert O.euler(len(rv), re_, rt) == O.ref_euler(rv, re_, rt)


def test_closed_pocket_survives():
    vts, edges, tris = octahedron_shell()
    rc = O.RefComplex(vts, edges, tris)
    r = O.thin(len(vts), edges, tris, np.zeros(rc.ne, np.float32), np.zeros(len(tris), np.float32), 1.0, 1.0)
    assert r["keep_f"].all()
    assert O.euler(*[len(vts), rc.edges(), tris])["euler"] == 2


@pytest.mark.parametrize("name,occ", [("torus40", None), ("grf32", None), ("csg", None)])
def test_lattice_vd_thin_vs_reference(name, occ):
    occ = {"torus40": lambda: volumes.torus_mesh(40), "grf32": lambda: volumes.grf(32, sigma=4.0, seed=11),
           "csg": lambda: volumes.csg(21, 20, 40)}[name]()
    L = lattice_case(O, occ)
    vd = L["vd"]
    rc = O.RefComplex(vd["vts"], vd["edges"], vd["tris"])
    assert rc.ne == len(vd["edges"])  # every triangle side is already an edge
    for t in (0.0, 0.04, 0.1, 0.5):
        thr = float(np.float32(np.float64(vd["inside_size"]) * t))
        r = O.thin(len(vd["vts"]), vd["edges"], vd["tris"], L["em_fin"], vd["fm"], thr, thr)
        ref = rc.thin(vd["vm"], L["em_fin"], vd["fm"], thr, thr)
        for key in ("keep_v", "keep_e", "keep_f", "removed_e"):
            assert np.array_equal(r[key], ref[key]), (t, key)


def _topology_cases():
    yield "octahedron", octahedron_shell()
    for seed in range(3):
        rng = np.random.default_rng(seed)
        yield f"grid{seed}", grid_surface(int(rng.integers(3, 12)), int(rng.integers(3, 12)), seed=seed)
    for name, occ in (("torus40", volumes.torus_mesh(40)), ("grf32", volumes.grf(32, sigma=4.0, seed=11)),
                      ("spheres40", volumes.spheres(40, count=12, seed=2)), ("csg", volumes.csg(21, 20, 40))):
        vd = lattice_case(O, occ)["vd"]
        yield name, (vd["vts"], vd["edges"], vd["tris"])


@pytest.mark.parametrize("name,cx", list(_topology_cases()), ids=[c[0] for c in _topology_cases()])
def test_closed_components_vs_reference(name, cx):
    """nClosedComponents: the oracle's restatement against the reference's own
    thinning, remainingCC() and compute_conn_cmpnts()."""
    vts, edges, tris = cx
    n = O.closed_components(len(vts), edges, tris)
    assert n == O.ref_closed_components(vts, edges, tris)
    if name == "octahedron":
        assert n == 1
