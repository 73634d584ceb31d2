"""The 512^3 workload itself, through properties that do not depend on the
size (the oracle's full thinning at this size takes minutes, so it is pinned
on the smaller cases of the other tests):
  * the site list equals the oracle's (extraction is linear, seconds on CPU);
  * the feature transform is exact at sampled lattice points (brute force over
    all sites in float64) and every site's own lattice point has d2 = 0;
  * simple-pair collapses preserve homotopy type, so the remaining complex has
    the Euler characteristic of the full complex;
  * two runs give identical results; the float measures are within 2^-24 of
    FP64; both feature-transform methods give the same transform."""
import hashlib

import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import volumes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grf512():
    return volumes.grf(512, sigma=6.0, seed=0)


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_full_size_properties(gpu_ctx, grf512):
    ctx = gpu_ctx
    occ = grf512
    r = ctx.run_plain(occ, 0.04)
    X, Y, Z = occ.shape
    # sites: the oracle's list, in order
    xyz_ref, _ = O.extract_sites(occ)
    sites = ctx.sites()
    assert r["n_sites"] == len(xyz_ref)
    assert np.array_equal(sites, xyz_ref)
    # feature transform: sampled points against brute force, ties to the lowest index
    d2, ids = ctx.ft()
    rng = np.random.default_rng(5)
    pts = np.stack([rng.integers(0, X + 1, 24), rng.integers(0, Y + 1, 24), rng.integers(0, Z + 1, 24)], 1)
    lat = (sites + 0.5).astype(np.int32)  # site coordinates on the corner lattice (exact)
    for a, b, c in pts:
        dd = (lat[:, 0] - a) ** 2 + (lat[:, 1] - b) ** 2 + (lat[:, 2] - c) ** 2
        best = dd.min()
        assert d2[a, b, c] == int(best)
        assert ids[a, b, c] == int(np.flatnonzero(dd == best)[0])
    li = (lat[:, 0].astype(np.int64) * (Y + 1) + lat[:, 1]) * (Z + 1) + lat[:, 2]
    assert (d2.reshape(-1)[li] == 0).all()
    # thinning preserves the Euler characteristic
    vd = r["vd"]
    chi_full = vd["nv"] - vd["ne"] + vd["nt"]
    eu = ctx.euler_remaining()
    assert eu["euler"] == chi_full, (eu, chi_full)
    rv, re_, rt = ctx.remaining_arrays()
    first = _digest(rv, re_, rt)
    fl = ctx.thin_flags()
    # deterministic: a second run gives the same remaining complex and flags
    r2 = ctx.run_plain(occ, 0.04)
    assert r2["rem"] == r["rem"] and r2["thin"] == r["thin"]
    assert _digest(*ctx.remaining_arrays()) == first
    fl2 = ctx.thin_flags()
    for k in fl:
        assert np.array_equal(fl[k], fl2[k]), k
    chk = ctx.lambda_fp64_check()
    assert chk["max_rel_err"] <= 2.0 ** -24 and chk["flips"] >= 0


def test_full_size_ft_methods_agree(gpu_ctx, grf512):
    """The window and envelope methods give the same transform at 512^3 (the
    window method is the one the autotuner keeps for this workload), and so
    the same remaining complex."""
    ctx = gpu_ctx
    occ = grf512
    try:
        out = {}
        for method in ("envelope", "window"):
            ctx.set_ft_method(method)
            r = ctx.run_plain(occ, 0.04)
            d2, ids = ctx.ft()
            out[method] = (_digest(d2, ids), r["rem"], _digest(*ctx.remaining_arrays()))
        assert out["envelope"] == out["window"]
    finally:
        ctx.set_ft_method("auto")
