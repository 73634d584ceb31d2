"""Regenerate tests/golden/golden_v1.npz from the reference's OWN compiled code.

Run from the repo root where the reference tree is available:
    python tests/golden/make_golden.py
It builds oracle/_ref/libvcref.so (the reference's ccthin.cpp,
cellcomplex.cpp, geomalgo.cpp, spaceinfo.cpp and surfacing.cpp against the
API shim) and records, for small seeded inputs:
  * Surfacer::extractBoundaryVts site lists (as lattice coordinates);
  * cellcomplex::finalize edge lists and face edge ids, and
    CellComplexThinning::prune survivor flags, remainingCC sizes and
    util::computeEulerChar, on (a) seeded generic complexes and (b) the
    lattice Voronoi complexes of small volumes (stored by volume + a SHA-256
    of the complex the reference thinned);
  * util::simpleTriangulate of polygons with 3..9 sides.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
from complexes import grid_surface, octahedron_shell, random_measures  # noqa: E402
from voxel_ma_gb300 import volumes  # noqa: E402

OUT = os.path.join(os.path.dirname(__file__), "golden_v1.npz")


def complex_hash(vts, edges, tris, em, fm) -> str:
    h = hashlib.sha256()
    for a in (vts, edges, tris, em, fm):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def golden_volumes():
    return {
        "torus32": volumes.torus_mesh(32),
        "grf24": volumes.grf(24, sigma=3.0, seed=7),
        "spheres28": volumes.spheres(28, count=6, seed=3),
        "csg11": volumes.csg(11, 12, 26),
        "edge_touch": edge_touch_volume(),
    }


def edge_touch_volume():
    """Voxels that touch the box faces, each other only by edges/corners, and a cavity."""
    o = np.zeros((9, 8, 7), np.uint8)
    o[0:3, 0:3, 0:3] = 1
    o[3, 3, 3] = 1          # corner-touching
    o[4:8, 4:8, 2:6] = 1
    o[5:7, 5:7, 3:5] = 0    # cavity
    o[8, 0, 6] = 1          # box corner voxel
    return o


def main():
    oracle.build(reference=True, tree=os.environ.get("VOXEL_MA_REFERENCE", "/root/reference"))
    out = {}
    # 1) site lists
    vols = golden_volumes()
    for name, occ in vols.items():
        s = oracle.ref_extract_sites(occ)
        out[f"vol_{name}"] = np.packbits(occ.ravel())
        out[f"shape_{name}"] = np.array(occ.shape, np.int32)
        out[f"sites_{name}"] = (s + 0.5).astype(np.int16)  # exact: sites are half-integers
    # 2) generic complexes
    cases = {
        "grid_a": grid_surface(12, 9, seed=1, drop=0.15, extra_edges=12),
        "grid_b": grid_surface(20, 16, seed=2, drop=0.05, extra_edges=30, unsorted=0.2, omit=0.1),
        "grid_c": grid_surface(7, 7, seed=3, drop=0.0, extra_edges=0, shuffle=False),
        "octa": octahedron_shell(),
    }
    for k, (vts, edges, tris) in cases.items():
        rc = oracle.RefComplex(vts, edges, tris)
        _, em, fm = random_measures(rc.ne, len(tris), seed=sum(k.encode()))
        for tag, thr in (("lo", 1.0), ("hi", 3.0)):
            r = rc.thin(np.zeros(len(vts), np.float32), em, fm, thr, thr)
            rv, re_, rt = rc.remaining()
            eu = oracle.ref_euler(rv, re_, rt)
            p = f"cc_{k}_{tag}_"
            out[p + "keep_v"] = np.packbits(r["keep_v"])
            out[p + "keep_e"] = np.packbits(r["keep_e"])
            out[p + "keep_f"] = np.packbits(r["keep_f"])
            out[p + "removed_e"] = np.packbits(r["removed_e"])
            out[p + "rem_sizes"] = np.array([len(rv), len(re_), len(rt)], np.int64)
            out[p + "rem_hash"] = np.frombuffer(hashlib.sha256(rv.tobytes() + re_.tobytes() + rt.tobytes())
                                                .digest(), np.uint8)
            out[p + "euler"] = np.array([eu["V"], eu["E"], eu["F"], eu["C"], eu["euler"]], np.int64)
            out[p + "thr"] = np.array([thr], np.float32)
        out[f"cc_{k}_vts"] = vts
        out[f"cc_{k}_edges"] = edges
        out[f"cc_{k}_tris"] = tris
        out[f"cc_{k}_em"] = em
        out[f"cc_{k}_fm"] = fm
        out[f"cc_{k}_fin_edges"] = rc.edges()
        out[f"cc_{k}_fin_tri_edges"] = rc.tri_edges()
    # 3) lattice Voronoi complexes of the volumes, thinned by the reference
    for name, occ in vols.items():
        xyz, li = oracle.extract_sites(occ)
        d2, ids = oracle.ft(occ.shape, li)
        vd = oracle.lattice_vd(occ, ids, xyz)
        rc = oracle.RefComplex(vd["vts"], vd["edges"], vd["tris"])
        em_fin = np.zeros(rc.ne, np.float32)
        em_fin[: len(vd["em"])] = vd["em"]
        for t in (0.04, 0.2):
            thr = float(np.float32(np.float64(vd["inside_size"]) * t))
            r = rc.thin(vd["vm"], em_fin, vd["fm"], thr, thr)
            rv, re_, rt = rc.remaining()
            eu = oracle.ref_euler(rv, re_, rt)
            p = f"vd_{name}_{t}_"
            out[p + "keep_v"] = np.packbits(r["keep_v"])
            out[p + "keep_e"] = np.packbits(r["keep_e"])
            out[p + "keep_f"] = np.packbits(r["keep_f"])
            out[p + "rem_sizes"] = np.array([len(rv), len(re_), len(rt)], np.int64)
            out[p + "euler"] = np.array([eu["V"], eu["E"], eu["F"], eu["C"], eu["euler"]], np.int64)
            out[p + "thr"] = np.array([thr], np.float32)
        out[f"vd_{name}_hash"] = np.frombuffer(bytes.fromhex(complex_hash(vd["vts"], vd["edges"], vd["tris"],
                                                                          vd["em"], vd["fm"])), np.uint8)
        out[f"vd_{name}_sizes"] = np.array([len(vd["vts"]), rc.ne, len(vd["tris"])], np.int64)
    # 4) simpleTriangulate
    R = oracle.ref()
    for n in range(3, 10):
        poly = np.arange(10, 10 + n, dtype=np.int32)
        tris = np.zeros((n - 2, 3), np.int32)
        R.vcref_simple_triangulate(n, poly.ctypes.data_as(oracle.c_vp), tris.ctypes.data_as(oracle.c_vp))
        out[f"tri_{n}"] = tris
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes,", len(out), "arrays")


if __name__ == "__main__":
    main()
