"""The CPU oracle reproduces the golden vectors recorded from the reference's
own compiled sources (tests/golden/make_golden.py).  Runs on any host."""
import numpy as np
import pytest

from complexes import random_measures  # noqa: F401
from helpers import complex_hash, golden_flags, golden_volume, golden_volume_names, lattice_case, rem_hash

CC_CASES = ["grid_a", "grid_b", "grid_c", "octa"]


@pytest.fixture(scope="module")
def O(oracle_lib):
    return oracle_lib


def test_sites_match_reference_golden(O, golden):
    for name in golden_volume_names(golden):
        occ = golden_volume(golden, name)
        xyz, _ = O.extract_sites(occ)
        ref = golden[f"sites_{name}"].astype(np.float32) - 0.5
        assert xyz.shape == ref.shape, name
        assert np.array_equal(xyz, ref), name


@pytest.mark.parametrize("case", CC_CASES)
def test_finalize_matches_reference_golden(O, golden, case):
    vts, edges, tris = (golden[f"cc_{case}_{k}"] for k in ("vts", "edges", "tris"))
    fin = O.finalize(len(vts), edges, tris)
    assert np.array_equal(fin["edges"], golden[f"cc_{case}_fin_edges"])
    assert np.array_equal(fin["tri_edges"], golden[f"cc_{case}_fin_tri_edges"])


@pytest.mark.parametrize("case", CC_CASES)
@pytest.mark.parametrize("tag", ["lo", "hi"])
def test_thin_matches_reference_golden(O, golden, case, tag):
    vts, edges, tris, em, fm = (golden[f"cc_{case}_{k}"] for k in ("vts", "edges", "tris", "em", "fm"))
    thr = float(golden[f"cc_{case}_{tag}_thr"][0])
    r = O.thin(len(vts), edges, tris, em, fm, thr, thr)
    assert r["rc"] == 0
    p = f"cc_{case}_{tag}_"
    for k, n in (("keep_v", len(vts)), ("keep_e", len(em)), ("keep_f", len(tris)), ("removed_e", len(em))):
        assert np.array_equal(r[k], golden_flags(golden, p + k, n)), k
    fin = O.finalize(len(vts), edges, tris)
    rv, re_, rt = O.remaining(vts, fin["edges"], tris, r["keep_v"], r["keep_e"], r["keep_f"])
    assert [len(rv), len(re_), len(rt)] == list(golden[p + "rem_sizes"])
    assert rem_hash(rv, re_, rt) == golden[p + "rem_hash"].tobytes()
    eu = O.euler(len(rv), re_, rt)
    assert [eu["V"], eu["E"], eu["F"], eu["C"], eu["euler"]] == list(golden[p + "euler"])


@pytest.mark.parametrize("name", ["torus32", "grf24", "spheres28", "csg11", "edge_touch"])
def test_lattice_vd_thin_matches_reference_golden(O, golden, name):
    occ = golden_volume(golden, name)
    L = lattice_case(O, occ)
    vd = L["vd"]
    assert complex_hash(vd["vts"], vd["edges"], vd["tris"], vd["em"], vd["fm"]) == \
        golden[f"vd_{name}_hash"].tobytes()
    for t in (0.04, 0.2):
        p = f"vd_{name}_{t}_"
        thr = float(golden[p + "thr"][0])
        assert thr == float(np.float32(np.float64(vd["inside_size"]) * t))
        r = O.thin(len(vd["vts"]), vd["edges"], vd["tris"], L["em_fin"], vd["fm"], thr, thr)
        assert r["rc"] == 0
        for k, n in (("keep_v", len(vd["vts"])), ("keep_e", len(L["em_fin"])), ("keep_f", len(vd["tris"]))):
            assert np.array_equal(r[k], golden_flags(golden, p + k, n)), (t, k)
        rv, re_, rt = O.remaining(vd["vts"], L["fin"]["edges"], vd["tris"], r["keep_v"], r["keep_e"], r["keep_f"])
        assert [len(rv), len(re_), len(rt)] == list(golden[p + "rem_sizes"])
        eu = O.euler(len(rv), re_, rt)
        assert [eu["V"], eu["E"], eu["F"], eu["C"], eu["euler"]] == list(golden[p + "euler"])


def test_simple_triangulate_golden(golden):
    # util::simpleTriangulate zig-zag order, restated
    for n in range(3, 10):
        poly = list(range(10, 10 + n))
        tris, i, j, inc = [], n - 1, 0, True
        while i - 1 > j:
            if inc:
                tris.append((poly[i], poly[j], poly[j + 1]))
                j += 1
            else:
                tris.append((poly[i], poly[j], poly[i - 1]))
                i -= 1
            inc = not inc
        assert np.array_equal(np.array(tris, np.int32), golden[f"tri_{n}"]), n


@pytest.mark.parametrize("vol", ["grf48", "torus64", "spheres96", "box_edge", "empty", "full"])
def test_lattice_vd_counts_match_the_complex(O, vol):
    """The counting restatement (used where the complex does not fit in host
    memory, the 1024^3 field) gives the sizes and inside size of the built
    complex."""
    from voxel_ma_gb300 import volumes
    if vol == "grf48":
        occ = volumes.grf(48, sigma=3.0, seed=5)
    elif vol == "torus64":
        occ = volumes.torus_mesh(64)
    elif vol == "spheres96":
        occ = volumes.spheres(96, count=12, seed=3)
    elif vol == "empty":
        occ = np.zeros((9, 11, 7), np.uint8)
    elif vol == "full":  # every voxel inside: sites on the box's surface only
        occ = np.ones((12, 9, 10), np.uint8)
    else:  # a box touching the volume's faces and edges
        occ = np.zeros((20, 17, 23), np.uint8)
        occ[:9, 4:, 3:21] = 1
    xyz, li = O.extract_sites(occ)
    _, ids = O.ft(occ.shape, li)
    vd = O.lattice_vd(occ, ids, xyz)
    cnt = O.lattice_vd_counts(occ, ids)
    assert [cnt["nv"], cnt["ne"], cnt["nt"]] == [len(vd["vts"]), len(vd["edges"]), len(vd["tris"])]
    assert cnt["nface"] == len(vd["face_sites"])
    assert cnt["inside_size"] == vd["inside_size"]
