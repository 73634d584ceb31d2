"""The feature transform's per-line envelope code (voxel_ma_gb300/csrc/
vc_ft_line.cuh) is the same source on the device and on the host: compiled
here with g++ and run on random lines (dense and sparse candidates, many
exact ties, rings small enough to force the spill path), it must equal a
brute-force lexicographic minimum at every point."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
SRC = os.path.join(ROOT, "tests", "cpp", "ft_line_check.cpp")


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_envelope_line_matches_brute_force(tmp_path):
    exe = str(tmp_path / "ft_line_check")
    subprocess.run(["g++", "-std=c++17", "-O2", SRC, "-o", exe], check=True, capture_output=True, text=True)
    r = subprocess.run([exe, "20000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
