"""The separable exact feature transform of the oracle equals brute force,
including the lowest-index tie-break, on small and degenerate volumes."""
import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import volumes


def _cases():
    rng = np.random.default_rng(5)
    yield "random", (rng.uniform(size=(9, 11, 13)) < 0.4).astype(np.uint8)
    yield "single", np.pad(np.ones((1, 1, 1), np.uint8), 2)
    yield "full", np.ones((5, 6, 7), np.uint8)
    yield "slab", np.pad(np.ones((2, 9, 9), np.uint8), ((3, 3), (0, 0), (0, 0)))
    yield "csg", volumes.csg(4, 10, 18)
    yield "spheres", volumes.spheres(20, count=5, seed=2)


@pytest.mark.parametrize("name,occ", list(_cases()))
def test_separable_equals_bruteforce(name, occ):
    xyz, li = O.extract_sites(occ)
    d2a, ida = O.ft(occ.shape, li, brute=True)
    for threads in (1, 3):
        d2b, idb = O.ft(occ.shape, li, threads=threads)
        assert np.array_equal(d2a, d2b), name
        assert np.array_equal(ida, idb), name


def test_empty_volume_has_no_sites():
    occ = np.zeros((6, 5, 4), np.uint8)
    xyz, li = O.extract_sites(occ)
    assert len(xyz) == 0
    d2, ids = O.ft(occ.shape, li)
    assert (ids == -1).all() and (d2 == np.iinfo(np.int32).max).all()


def test_ties_go_to_lowest_index():
    # two sites equidistant from the centre point of a 1-voxel gap
    occ = np.zeros((3, 1, 1), np.uint8)
    occ[0] = 1
    occ[2] = 1
    xyz, li = O.extract_sites(occ)
    d2, ids = O.ft(occ.shape, li)
    d2b, idb = O.ft(occ.shape, li, brute=True)
    assert np.array_equal(ids, idb) and np.array_equal(d2, d2b)


@pytest.mark.parametrize("name,occ", list(_cases())[:3])
def test_radius_follows_the_reference_loop(name, occ):
    """VoroInfo::computeInfoRelatedtoSites (voroinfo.cpp:286-325) restated as
    a plain loop: every Voronoi face, in face order, writes the distance from
    its first site to each of its vertices; the last write wins."""
    xyz, li = O.extract_sites(occ)
    _, ids = O.ft(occ.shape, li)
    vd = O.lattice_vd(occ, ids, xyz)
    X, Y, Z = occ.shape
    vid = {tuple(int(c) for c in v): i for i, v in enumerate(vd["vts"])}
    r = np.zeros(len(vd["vts"]), np.float32)
    for a in range(X + 1):
        for b in range(Y + 1):
            for c in range(Z + 1):
                for d in range(3):
                    e = [a, b, c]
                    e[d] += 1
                    if e[0] > X or e[1] > Y or e[2] > Z:
                        continue
                    s0, s1 = ids[a, b, c], ids[e[0], e[1], e[2]]
                    if s0 < 0 or s1 < 0 or s0 == s1:
                        continue
                    u, w = (d + 1) % 3, (d + 2) % 3
                    for s, t in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        v = [0, 0, 0]
                        v[d], v[u], v[w] = (a, b, c)[d], (a, b, c)[u] - 1 + s, (a, b, c)[w] - 1 + t
                        i = vid.get(tuple(v))
                        if i is None:
                            continue
                        diff = np.float32(v) - xyz[s0]
                        acc = np.float32(0)
                        for k in range(3):
                            acc = np.float32(acc + np.float32(diff[k] * diff[k]))
                        r[i] = np.sqrt(acc, dtype=np.float32)
    assert len(vd["radius"]) == len(vd["vts"])
    assert np.array_equal(vd["radius"], r)
    # every vertex lies on some Voronoi face, so every radius was written
    assert (vd["radius"] > 0).all() or len(r) == 0
