"""The full-size workloads, bit for bit: the 64^3 torus, the 32-sphere unions at
256^3 (seeds 0, 1, 2) and the 512^3 thresholded random field that the
benchmark times; at 1024^3, the sites, the feature transform and the
complex's sizes and threshold (the rest of the path there by its properties).

The CPU oracle's outputs at these sizes take minutes and tens of GB of host
memory, so tests/golden/make_fullsize_digests.py ran it once and committed
sha256 digests of every stage (tests/golden/fullsize_digests.json); for the
torus and the sphere unions it also ran the reference's own compiled thinning
and remainingCC on the same complex and checked that they agree.  Here the GPU
path runs on the same volumes (their occupancy digests are checked first) and
every stage must give the same bytes: sites in order, squared distances and
nearest-site ids of the feature transform, the lattice complex with its
measures, the threshold, the thinning's queue statistics, the surviving
vertex / edge / face flags and removed-edge flags, the remaining arrays and
their Euler characteristic.

Properties that do not need the oracle are checked on the 512^3 field too:
simple-pair collapses preserve the Euler characteristic, reruns are
identical, both feature-transform methods agree, and the float measures are
within 2^-24 of FP64."""
import hashlib
import json
import os

import numpy as np
import pytest

from voxel_ma_gb300 import volumes

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
DIGESTS = json.load(open(os.path.join(HERE, "golden", "fullsize_digests.json")))


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _flags01(a):
    return (np.asarray(a) != 0).astype(np.uint8)


def _volume(name):
    import torch
    if name == "torus64":
        return volumes.torus_mesh(64)
    if name.startswith("spheres256_s"):
        return volumes.spheres(256, count=32, seed=int(name[len("spheres256_s"):]))
    if name in ("grf512", "grf1024"):
        return volumes.grf(int(name[3:]), sigma=6.0, seed=0, device=torch.device("cuda"))
    raise KeyError(name)


FULL = sorted(k for k, v in DIGESTS.items() if "stages" not in v)
FT_ONLY = sorted(k for k, v in DIGESTS.items() if v.get("stages", "").startswith("sites+ft"))


@pytest.fixture(scope="module")
def grf512():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    occ = _volume("grf512")
    assert volumes.occupancy_sha256(occ) == volumes.WORKLOAD_SHA256["grf512_sigma6_level0"]
    return occ


@pytest.mark.parametrize("name", FT_ONLY)
def test_full_path_at_1024(name):
    """The 1024^3 field (1.08e9 lattice points, 1.24e8 sites; a complex of
    about 5e8 vertices, 2.1e9 edges and 1.6e9 triangles).  Site list and
    feature transform bit for bit against the oracle's digests, and the
    complex's sizes, inside size and threshold against the oracle's count of
    them; the oracle's complex at this size does not fit the host it ran on,
    so the rest is checked by properties: the queue positions pass 2^31 (V +
    E > 2^31), the processed pairs are the pushes less the skips, simple-pair
    collapses keep the Euler characteristic, and a second run gives the same
    thinning and the same remaining complex.  (The same kernels are pinned to the oracle
    at 512^3 above, and with positions above 2^31 and the queue capacity at
    its limit in test_gpu_thin_queue.py.)"""
    import torch
    from voxel_ma_gb300 import api
    d = DIGESTS[name]
    occ = _volume(name)
    assert volumes.occupancy_sha256(occ) == d["occupancy_sha256"]
    torch.cuda.empty_cache()  # the field's blur temporaries
    with api.Context(0) as ctx:
        r = ctx.run_plain(occ, 0.04)
        assert r["n_sites"] == d["n_sites"]
        assert _digest(ctx.sites()) == d["sites"]
        assert _digest(*ctx.ft()) == d["ft"]
        vd = r["vd"]
        if "vd_sizes" in d:
            assert [vd["nv"], vd["ne"], vd["nt"]] == d["vd_sizes"]
            assert vd["inside_size"] == d["inside_size"] and r["thresh"] == d["thresh"]
        assert vd["nv"] + vd["ne"] > 2**31, vd
        th = r["thin"]
        assert th["pushes"] - th["skipped"] == th["processed"] > 0
        eu = ctx.euler_remaining()
        assert eu["euler"] == vd["nv"] - vd["ne"] + vd["nt"], (eu, vd)
        first = _digest(*ctx.remaining_arrays())
        r2 = ctx.run_plain(occ, 0.04)
        assert r2 == r
        assert _digest(*ctx.remaining_arrays()) == first


@pytest.mark.parametrize("name", FULL)
def test_full_size_stages_bit_exact(gpu_ctx, name):
    ctx = gpu_ctx
    d = DIGESTS[name]
    occ = _volume(name)
    assert volumes.occupancy_sha256(occ) == d["occupancy_sha256"], "not the volume the digests were made from"
    r = ctx.run_plain(occ, d["t"])
    assert r["n_sites"] == d["n_sites"]
    assert _digest(ctx.sites()) == d["sites"], "site list"
    assert _digest(*ctx.ft()) == d["ft"], "feature transform"
    assert [r["vd"]["nv"], r["vd"]["ne"], r["vd"]["nt"]] == d["vd_sizes"]
    assert r["vd"]["inside_size"] == d["inside_size"]
    assert r["thresh"] == d["thresh"]
    # the pairs popped and processed (the GPU drops, instead of pushing, a
    # child whose cell goes in the same generation: the reference pops and
    # skips it, so pushes, skips and a trailing generation of skips only can
    # differ while the processed pairs match)
    assert r["thin"]["processed"] == d["thin_stats"]["processed"]
    assert r["thin"]["pushes"] - r["thin"]["skipped"] == r["thin"]["processed"]
    assert r["thin"]["generations"] <= d["thin_stats"]["generations"]
    fl = ctx.thin_flags()
    for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
        assert _digest(_flags01(fl[k])) == d[k], k
    del fl
    assert [r["rem"]["nv"], r["rem"]["ne"], r["rem"]["nt"]] == d["remaining_sizes"]
    assert _digest(*ctx.remaining_arrays()) == d["remaining"], "remaining arrays"
    assert ctx.euler_remaining() == d["remaining_euler"]
    vd = ctx.vd()
    assert _digest(vd["vts"], vd["edges"], vd["tris"], vd["em"], vd["fm"]) == d["complex"], "lattice complex"


def test_full_size_properties(gpu_ctx, grf512):
    ctx = gpu_ctx
    occ = grf512
    r = ctx.run_plain(occ, 0.04)
    # thinning preserves the Euler characteristic
    vd = r["vd"]
    chi_full = vd["nv"] - vd["ne"] + vd["nt"]
    eu = ctx.euler_remaining()
    assert eu["euler"] == chi_full, (eu, chi_full)
    first = _digest(*ctx.remaining_arrays())
    fl = ctx.thin_flags()
    # deterministic: a second run gives the same remaining complex and flags
    r2 = ctx.run_plain(occ, 0.04)
    assert r2["rem"] == r["rem"] and r2["thin"] == r["thin"]
    assert _digest(*ctx.remaining_arrays()) == first
    fl2 = ctx.thin_flags()
    for k in fl:
        assert np.array_equal(fl[k], fl2[k]), k
    chk = ctx.lambda_fp64_check()
    assert chk["max_rel_err"] <= 2.0 ** -24 and chk["flips"] == 0


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
            out[method] = (_digest(*ctx.ft()), r["rem"], _digest(*ctx.remaining_arrays()))
        assert out["envelope"] == out["window"]
        assert out["window"][0] == DIGESTS["grf512"]["ft"]
    finally:
        ctx.set_ft_method("auto")
