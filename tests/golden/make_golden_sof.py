"""Regenerate tests/golden/golden_sof.npz from the reference's OWN compiled code.

Run from the repo root where the reference tree is available:
    python tests/golden/make_golden_sof.py
It builds oracle/_ref/libvcref.so (which includes the reference's octree.cpp)
and records, for small seeded volumes:
  * the .sof file the reference writes for the volume (OctreeVolume built
    from the dense volume, then writeToFile);
  * the .sog file it writes for the same octree (write_sog_file), and its
    reading of that file;
  * the reference's reading of the .sof file: the occupancy of every voxel of
    its (R+1)^3 grid (SpaceConverter::get_occupancy_at_vox on the octree)
    and the sites of Surfacer::extractBoundaryVts on it (its octree branch),
    stored as lattice coordinates (site + 0.5).
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from voxel_ma_gb300 import volumes  # noqa: E402

OUT = os.path.join(os.path.dirname(__file__), "golden_sof.npz")


def sof_volumes():
    rng = np.random.default_rng(17)
    return {
        "torus40": volumes.torus_mesh(40),
        "grf32": volumes.grf(32, sigma=4.0, seed=5),
        "spheres30": volumes.spheres(30, count=5, seed=8),
        "csg13": volumes.csg(13, 14, 30),
        "noise": (rng.uniform(size=(9, 14, 6)) < 0.5).astype(np.uint8),
    }


def main():
    oracle.build(reference=True, tree=os.environ.get("VOXEL_MA_REFERENCE", "/root/reference"))
    out = {}
    with tempfile.TemporaryDirectory() as d:
        for name, occ in sof_volumes().items():
            path = os.path.join(d, f"{name}.sof")
            oracle.ref_sof_write(np.asarray(occ), path)
            data = np.frombuffer(open(path, "rb").read(), np.uint8)
            occ_ref, sites_ref = oracle.ref_sof_read(path)
            out[f"sof_{name}"] = data
            out[f"sofocc_{name}"] = np.packbits(occ_ref.ravel())
            out[f"sofsize_{name}"] = np.array([occ_ref.shape[0]], np.int32)
            out[f"sofsites_{name}"] = (sites_ref + 0.5).astype(np.int16)
            # the same octree as .sog (write_sog_file / read_sog_file); bytes
            # 31..127 of its header are left uninitialised by the reference
            path = os.path.join(d, f"{name}.sog")
            oracle.ref_sof_write(np.asarray(occ), path)
            data = np.frombuffer(open(path, "rb").read(), np.uint8)
            occ_ref, sites_ref = oracle.ref_sof_read(path)
            out[f"sog_{name}"] = data
            out[f"sogocc_{name}"] = np.packbits(occ_ref.ravel())
            out[f"sogsites_{name}"] = (sites_ref + 0.5).astype(np.int16)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


if __name__ == "__main__":
    main()
