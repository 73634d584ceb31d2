"""The C++ adapters (include/voxelcore_gb300.hpp) keep the reference's class
surfaces; a driver written like exportInsideVoroMesh compiles against them
and, on a GPU, reproduces the oracle's surviving cell set."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
SRC = os.path.join(ROOT, "tests", "cpp", "adapter_main.cpp")
DROPIN = os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp")


def _compile(out, syntax_only=False, src=SRC):
    from voxel_ma_gb300 import _lib
    _lib.load()  # builds the library if needed
    cmd = ["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), src]
    if syntax_only:
        cmd += ["-fsyntax-only"]
    else:
        libdir = os.path.join(ROOT, "voxel_ma_gb300")
        cmd += ["-o", out, "-L" + libdir, "-lvoxelcore_gb300", "-Wl,-rpath," + libdir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_adapter_header_compiles():
    _compile(None, syntax_only=True)
    _compile(None, syntax_only=True, src=DROPIN)


def _write_volume(path, occ):
    with open(path, "wb") as f:
        f.write(np.array(occ.shape, np.int32).tobytes())
        f.write(np.ascontiguousarray(occ).tobytes())


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_reference_style_caller_runs_unchanged(tmp_path):
    """tests/cpp/dropin_main.cpp calls Surfacer, VoroInfo, cellcomplex,
    CellComplexThinning (both remainingCC forms) and nClosedComponents as the
    reference's own callers do, with no GPU context in sight; its results are
    the oracle's."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oracle
    from voxel_ma_gb300 import volumes
    exe = str(tmp_path / "dropin_main")
    _compile(exe, src=DROPIN)
    occ = volumes.csg(11, 24, 40)
    vol = tmp_path / "vol.bin"
    _write_volume(vol, occ)
    t = 0.04
    from mrc_files import value_volume, write_mrc
    mrc = tmp_path / "vol.mrc"
    mrc.write_bytes(write_mrc(value_volume(occ, 2), 2, axes=(3, 1, 2)))
    run = subprocess.run([exe, str(vol), str(t), str(mrc)], capture_output=True, text=True)
    assert run.returncode == 0, run.stderr
    out = run.stdout
    lines = dict(line.split(" ", 1) if " " in line else (line, "") for line in out.strip().splitlines())
    ref = oracle.run_plain(occ, t=t)
    vd = ref["vd"]
    assert int(lines["sites"]) == len(ref["sites"])
    assert np.float32(float(lines["thresh"])) == np.float32(ref["thresh"])
    assert [int(x) for x in lines["complex"].split()] == [len(vd["vts"]), len(ref["fin"]["edges"]), len(vd["tris"])]
    keep_f = np.nonzero(ref["thin"]["keep_f"])[0]
    assert np.array_equal(np.array(lines["keep_f"].split(), np.int64), keep_f)
    assert np.array_equal(np.array(lines["from_fi"].split(), np.int64), keep_f)
    assert np.array_equal(np.array(lines["rem_tris"].split(), np.int32).reshape(-1, 3), ref["rem_tris"])
    assert np.array_equal(np.array(lines["rem_edges"].split(), np.int32).reshape(-1, 2), ref["rem_edges"])
    nv, ne, nt = (int(x) for x in lines["remaining"].split())
    assert (nv, ne, nt) == (len(ref["rem_vts"]), len(ref["rem_edges"]), len(ref["rem_tris"]))
    cv, ce, ct = (int(x) for x in lines["remaining_cc"].split())
    assert (cv, ct) == (nv, nt) and ce == len(oracle.finalize_edges(nv, ref["rem_edges"], ref["rem_tris"]))
    assert int(lines["closed"]) == oracle.closed_components(len(vd["vts"]), vd["edges"], vd["tris"])
    assert int(lines["radii"]) == len(vd["vts"])
    assert int(lines["file_sites"]) == len(ref["sites"])
    assert [int(x) for x in lines["file_complex"].split()] == [len(vd["vts"]), len(vd["edges"]), len(vd["tris"])]


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
@pytest.mark.parametrize("t", [0.04, 0.2])
def test_adapter_drives_gpu_path_like_the_reference(tmp_path, t):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import oracle
    from voxel_ma_gb300 import volumes
    exe = str(tmp_path / "adapter_main")
    _compile(exe)
    occ = volumes.csg(7, 24, 40)
    vol = tmp_path / "vol.bin"
    with open(vol, "wb") as f:
        f.write(np.array(occ.shape, np.int32).tobytes())
        f.write(np.ascontiguousarray(occ).tobytes())
    out = subprocess.run([exe, str(vol), str(t)], check=True, capture_output=True, text=True).stdout
    lines = dict(line.split(" ", 1) if " " in line else (line, "") for line in out.strip().splitlines())
    ref = oracle.run_plain(occ, t=t)
    assert int(lines["sites"]) == len(ref["sites"])
    assert np.float32(float(lines["thresh"])) == np.float32(ref["thresh"])
    for key in ("keep_v", "keep_e", "keep_f"):
        got = np.array([int(x) for x in lines[key].split()], np.int64)
        assert np.array_equal(got, np.nonzero(ref["thin"][key])[0]), key
    from helpers import lattice_case
    radius = np.array([float(x) for x in lines["radius"].split()], np.float32)
    assert np.array_equal(radius, lattice_case(oracle, occ)["vd"]["radius"])
    nv, ne, nt = (int(x) for x in lines["remaining"].split())
    assert (nv, ne, nt) == (len(ref["rem_vts"]), len(ref["rem_edges"]), len(ref["rem_tris"]))


@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_export_adapters_write_the_library_bytes(tmp_path):
    """vcgpu::writeToPLY / writeToDotma / writeOctreeFile (host code, no GPU)
    write the same bytes as the library's C entry points."""
    from voxel_ma_gb300 import _lib, api
    _lib.load()
    exe = str(tmp_path / "export_main")
    libdir = os.path.join(ROOT, "voxel_ma_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "export_main.cpp"), "-o", exe, "-L" + libdir,
                    "-lvoxelcore_gb300", "-Wl,-rpath," + libdir], check=True, capture_output=True, text=True)
    rng = np.random.default_rng(4)
    nv, ne, nt = 500, 60, 700
    vts = rng.uniform(-10, 600, (nv, 3)).astype(np.float32)
    radii = rng.uniform(0, 30, nv).astype(np.float32)
    edges = rng.integers(0, nv, (ne, 2)).astype(np.int32)
    tris = rng.integers(0, nv, (nt, 3)).astype(np.int32)
    blob = tmp_path / "complex.bin"
    with open(blob, "wb") as f:
        f.write(np.array([nv, ne, nt], np.int64).tobytes())
        for a in (vts, radii, edges, tris):
            f.write(np.ascontiguousarray(a).tobytes())
    prefix = str(tmp_path / "cpp")
    subprocess.run([exe, str(blob), prefix], check=True, capture_output=True, text=True)
    api.write_ply(str(tmp_path / "py.ply"), vts, edges, tris)
    api.write_dotma(str(tmp_path / "py.ma"), vts, radii, edges, tris)
    for ext in (".ply", ".ma"):
        assert open(prefix + ext, "rb").read() == open(str(tmp_path / "py") + ext, "rb").read(), ext
    occ = np.ones((9, 7, 5), np.uint8)
    occ[4, 3, 2] = 0
    assert open(prefix + ".sof", "rb").read() == api.encode_sof(occ)
    assert open(prefix + ".sog", "rb").read() == api.encode_sog(occ)
