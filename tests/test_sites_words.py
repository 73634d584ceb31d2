"""The word-parallel site rule (voxel_ma_gb300/csrc/vc_sites_words.cuh) is
the same source on the device and on the host: compiled here with g++, it
must give the oracle's site list, in the reference's order, on volumes with
every kind of boundary (box faces, word edges at z = 31/32/33, rows shorter
than a word, thin and empty volumes)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import volumes

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
SRC = os.path.join(ROOT, "tests", "cpp", "sites_words_check.cpp")


def _cases():
    rng = np.random.default_rng(5)
    yield "torus64", volumes.torus_mesh(64)
    yield "spheres96", volumes.spheres(96, count=32, seed=1)
    yield "grf40", volumes.grf(40, sigma=3.0, seed=2)
    for shape in [(3, 4, 31), (2, 3, 32), (3, 2, 33), (1, 1, 1), (1, 5, 70), (4, 4, 64), (5, 3, 97)]:
        for p in (0.2, 0.5, 0.9):
            yield f"noise{shape}_{p}", (rng.uniform(size=shape) < p).astype(np.uint8)
    yield "full", np.ones((3, 4, 40), np.uint8)
    yield "empty", np.zeros((3, 4, 40), np.uint8)


CASES = list(_cases())


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("sw") / "sites_words_check")
    subprocess.run(["g++", "-std=c++17", "-O2", SRC, "-o", out], check=True, capture_output=True, text=True)
    return out


@pytest.mark.parametrize("name,occ", CASES, ids=[c[0] for c in CASES])
def test_word_rule_matches_oracle(exe, tmp_path, oracle_lib, name, occ):
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        f.write(np.asarray(occ.shape, np.int32).tobytes())
        f.write(occ.tobytes())
    subprocess.run([exe, str(fin), str(fout)], check=True, timeout=120)
    raw = open(fout, "rb").read()
    n = int(np.frombuffer(raw[:8], np.int64)[0])
    pts = np.frombuffer(raw[8:], np.int32).reshape(n, 3)
    xyz, _ = O.extract_sites(occ)
    assert n == len(xyz)
    assert np.array_equal(pts.astype(np.float32) - 0.5, xyz)
