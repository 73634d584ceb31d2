"""Output formats of the remaining complex: vc_write_ply, vc_write_radii,
vc_write_dotma and vc_dotma_edges (host code of the library, no GPU) against
the oracle restatement on std::ofstream / stdio, and, where the reference tree
was built here, against the reference's own writeToDotma
(src/exporters.cpp:244-287) and its .ma edge assembly on its own ivec2Hash
(src/highlevelalgo.cpp:925-937)."""
import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import _lib, api


def _complex(seed, nv=400, ne=120, nt=600, id_scale=1):
    rng = np.random.default_rng(seed)
    kinds = rng.integers(0, 6, size=(nv, 3))
    vals = np.select(
        [kinds == 0, kinds == 1, kinds == 2, kinds == 3, kinds == 4],
        [rng.uniform(0, 512, (nv, 3)), rng.integers(0, 512, (nv, 3)) + 0.5, rng.uniform(-1e-4, 1e-4, (nv, 3)),
         rng.uniform(1e5, 1e8, (nv, 3)), -rng.uniform(0, 600, (nv, 3))],
        rng.integers(0, 512, (nv, 3)).astype(np.float64))
    vts = vals.astype(np.float32)
    radii = np.abs(rng.normal(3.0, 4.0, nv)).astype(np.float32)
    radii[:5] = [0.0, 0.5, 1e-3, 1234567.0, np.float32(np.sqrt(2.0))]
    edges = rng.integers(0, nv, size=(ne, 2)).astype(np.int32) * id_scale
    a = rng.integers(0, nv, nt)
    d1 = rng.integers(1, nv - 1, nt)
    d2 = d1 + rng.integers(1, nv - d1, nt)             # 0 < d1 < d2 < nv: three distinct ids
    tris = (np.stack([a, (a + d1) % nv, (a + d2) % nv], 1) * id_scale).astype(np.int32)
    return vts, radii, edges, tris


@pytest.mark.parametrize("seed", range(3))
def test_dotma_ply_radii_bytes_match_the_oracle(tmp_path, seed):
    vts, radii, edges, tris = _complex(seed)
    for kind in ("ma", "ply", "r"):
        a, b = str(tmp_path / f"a.{kind}"), str(tmp_path / f"b.{kind}")
        if kind == "ma":
            api.write_dotma(a, vts, radii, edges, tris)
            O.write_dotma(b, vts, radii, edges, tris)
        elif kind == "ply":
            api.write_ply(a, vts, edges, tris)
            O.write_ply(b, vts, edges, tris)
        else:
            api.write_radii(a, vts, radii)
            O.write_radii(b, vts, radii)
        assert open(a, "rb").read() == open(b, "rb").read(), kind


@pytest.mark.skipif(not O.ref_available(), reason="the reference's sources are not built on this host")
@pytest.mark.parametrize("seed", range(3))
def test_dotma_bytes_match_the_reference(tmp_path, seed):
    vts, radii, edges, tris = _complex(seed)
    a, b = str(tmp_path / "a.ma"), str(tmp_path / "b.ma")
    api.write_dotma(a, vts, radii, edges, tris)
    O.ref_write_dotma(b, vts, radii, edges, tris)
    assert open(a, "rb").read() == open(b, "rb").read()


@pytest.mark.parametrize("seed,scale", [(0, 1), (1, 1), (2, 997), (3, 65537)])
def test_dotma_edge_order(seed, scale):
    # thousands of triangle edges: the set rehashes several times
    _, _, edges, tris = _complex(seed, nv=2000, ne=50, nt=5000, id_scale=scale)
    got = api.dotma_edges(edges, tris)
    assert np.array_equal(got, O.dotma_edges(edges, tris))
    assert np.array_equal(got[: len(edges)], edges)
    if O.ref_available():
        assert np.array_equal(got, O.ref_dotma_edges(edges, tris))


def test_empty_complex_and_errors(tmp_path):
    z3f, z2i, z3i = np.zeros((0, 3), np.float32), np.zeros((0, 2), np.int32), np.zeros((0, 3), np.int32)
    for kind in ("ma", "ply", "r"):
        a, b = str(tmp_path / f"a.{kind}"), str(tmp_path / f"b.{kind}")
        if kind == "ma":
            api.write_dotma(a, z3f, [], z2i, z3i)
            O.write_dotma(b, z3f, [], z2i, z3i)
        elif kind == "ply":
            api.write_ply(a, z3f, z2i, z3i)
            O.write_ply(b, z3f, z2i, z3i)
        else:
            api.write_radii(a, z3f, [])
            O.write_radii(b, z3f, [])
        assert open(a, "rb").read() == open(b, "rb").read(), kind
    assert len(api.dotma_edges(z2i, z3i)) == 0
    with pytest.raises(_lib.VoxelCoreError) as ei:
        api.write_ply(str(tmp_path / "missing_dir" / "x.ply"), z3f, z2i, z3i)
    assert ei.value.status == _lib.VC_ERR_ARG
    with pytest.raises(ValueError):
        api.write_radii(str(tmp_path / "x.r"), np.zeros((2, 3), np.float32), [1.0])


def test_large_inputs_use_several_threads(tmp_path):
    # enough lines and edges that the formatting and the edge de-duplication
    # run on several threads; the bytes and the order must not change
    vts, radii, edges, tris = _complex(9, nv=150_000, ne=20_000, nt=120_000)
    got = api.dotma_edges(edges, tris)
    assert np.array_equal(got, O.dotma_edges(edges, tris))
    if O.ref_available():
        assert np.array_equal(got, O.ref_dotma_edges(edges, tris))
    for kind in ("ma", "ply", "r"):
        a, b = str(tmp_path / f"a.{kind}"), str(tmp_path / f"b.{kind}")
        if kind == "ma":
            api.write_dotma(a, vts, radii, got, tris)
            O.write_dotma(b, vts, radii, got, tris)
        elif kind == "ply":
            api.write_ply(a, vts, edges, tris)
            O.write_ply(b, vts, edges, tris)
        else:
            api.write_radii(a, vts, radii)
            O.write_radii(b, vts, radii)
        assert open(a, "rb").read() == open(b, "rb").read(), kind
