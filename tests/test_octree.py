"""Octree (.sof) volumes: the oracle's decoding against the fixtures the
reference's own octree code wrote and read (tests/golden/golden_sof.npz,
made by tests/golden/make_golden_sof.py), and against the reference itself
on fresh volumes where its tree is present."""
import os
import tempfile

import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import volumes

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


@pytest.fixture(scope="module")
def sof_golden():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "golden_sof.npz")))


def sof_names(g):
    return sorted(k[len("sof_"):] for k in g if k.startswith("sof_"))


def test_oracle_decodes_reference_files(oracle_lib, sof_golden):
    g = sof_golden
    for name in sof_names(g):
        occ, sites = O.sof_decode(g[f"sof_{name}"].tobytes())
        n = int(g[f"sofsize_{name}"][0])
        assert occ.shape == (n, n, n), name
        assert np.array_equal(np.packbits(occ.ravel()), g[f"sofocc_{name}"]), name
        assert np.array_equal(sites, g[f"sofsites_{name}"].astype(np.float32) - 0.5), name


def test_malformed_streams_are_rejected(oracle_lib, sof_golden):
    data = sof_golden["sof_grf32"].tobytes()
    assert O.sof_decode(data[:-3]) is None                       # truncated
    assert O.sof_decode(np.int32(24).tobytes() + data[4:]) is None  # resolution not a power of two
    bad = bytearray(data)
    bad[4] = 7                                                  # unknown node type
    assert O.sof_decode(bytes(bad)) is None
    assert O.sof_decode(b"\x01") is None


@pytest.mark.skipif(not O.ref_available() and not O.reference_tree_present(),
                    reason="reference tree not present on this host")
@pytest.mark.parametrize("seed", range(4))
def test_oracle_vs_reference_fresh_volumes(oracle_lib, seed):
    rng = np.random.default_rng(300 + seed)
    shape = tuple(int(s) for s in rng.integers(3, 40, 3))
    occ = (rng.uniform(size=shape) < rng.uniform(0.2, 0.8)).astype(np.uint8)
    if seed == 3:
        occ = volumes.csg(40 + seed, 10, 36)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "v.sof")
        O.ref_sof_write(occ, path)
        occ_ref, sites_ref = O.ref_sof_read(path)
        occ_o, sites_o = O.sof_decode(open(path, "rb").read())
    assert np.array_equal(occ_o, occ_ref)
    assert np.array_equal(sites_o, sites_ref)
    # the octree holds the volume: its voxels beyond the volume are outside
    S = occ_ref.shape[0]
    emb = np.zeros((S, S, S), np.uint8)
    emb[: occ.shape[0], : occ.shape[1], : occ.shape[2]] = occ > 0
    assert np.array_equal(occ_o, emb)


def _golden_sof_volumes():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden_sof", os.path.join(ROOT, "tests", "golden", "make_golden_sof.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.sof_volumes()


def test_encoder_writes_the_reference_bytes(sof_golden):
    """vc_encode_sof (host code of the library, no GPU) against the files the
    reference's OctreeVolume wrote for the same volumes."""
    from voxel_ma_gb300 import api
    for name, occ in _golden_sof_volumes().items():
        assert api.encode_sof(np.asarray(occ)) == sof_golden[f"sof_{name}"].tobytes(), name


@pytest.mark.parametrize("seed", range(6))
def test_encode_decode_round_trip(oracle_lib, seed):
    from voxel_ma_gb300 import api
    rng = np.random.default_rng(500 + seed)
    shape = tuple(int(s) for s in rng.integers(1, 34, 3))
    occ = (rng.uniform(size=shape) < rng.uniform(0.1, 0.9)).astype(np.uint8)
    occ_d, _ = O.sof_decode(api.encode_sof(occ))
    S = occ_d.shape[0]
    emb = np.zeros((S, S, S), np.uint8)
    emb[: shape[0], : shape[1], : shape[2]] = occ
    assert np.array_equal(occ_d, emb)
    if O.ref_available():
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "v.sof")
            O.ref_sof_write(occ, path)
            assert open(path, "rb").read() == api.encode_sof(occ)
    occ_g, _ = O.sof_decode(api.encode_sog(occ), sog=True)
    assert np.array_equal(occ_g, emb)


SOG_NAMES = ["csg13", "grf32", "noise", "spheres30", "torus40"]


@pytest.mark.parametrize("name", SOG_NAMES)
def test_sog_oracle_and_encoder_match_the_reference(sof_golden, name):
    """.sog files written and read by the reference (write_sog_file /
    read_sog_file): the oracle's decoding equals the reference's reading, and
    vc_encode_sog writes the same bytes, but for the header bytes 31..127 the
    reference leaves uninitialised."""
    g = sof_golden
    data = g[f"sog_{name}"].tobytes()
    occ, sites = O.sof_decode(data, sog=True)
    assert np.array_equal(np.packbits(occ.ravel()), g[f"sogocc_{name}"])
    assert np.array_equal((sites + 0.5).astype(np.int16), g[f"sogsites_{name}"])
    assert np.array_equal(g[f"sogocc_{name}"], g[f"sofocc_{name}"])  # same octree as the .sof


def test_sog_encoder_bytes(sof_golden):
    from voxel_ma_gb300 import api
    for name, occ in _golden_sof_volumes().items():
        ref = sof_golden[f"sog_{name}"].tobytes()
        enc = api.encode_sog(np.asarray(occ))
        assert len(enc) == len(ref), name
        assert enc[:31] == ref[:31] and enc[128:] == ref[128:], name
        assert enc[31:128] == bytes(97)


def test_malformed_sog_is_rejected_by_the_oracle(sof_golden):
    data = sof_golden["sog_grf32"].tobytes()
    assert O.sof_decode(data[:-5], sog=True) is None           # truncated inside a leaf's feature point
    assert O.sof_decode(b"SOG.Format 2.0\0" + data[15:], sog=True) is None
    assert O.sof_decode(data[:100], sog=True) is None
