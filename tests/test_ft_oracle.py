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
