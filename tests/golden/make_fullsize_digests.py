"""Writes tests/golden/fullsize_digests.json: sha256 digests of every stage of
the CPU oracle on the full-size workloads, for the GPU tests to compare with
(tests/test_gpu_fullsize.py).  Those runs take minutes and tens of GB of host
memory at 512^3, too much for a test, so they are made once here.

Workloads:
  torus64        the closed triangle-mesh torus voxelized to 64^3;
  spheres256_s*  unions of 32 spheres at 256^3, seeds 0, 1, 2;
  grf512         the thresholded smoothed random field at 512^3 (sigma 6,
                 level 0, seed 0): the benchmark's own workload;
  grf1024        the same field at 1024^3: sites and feature transform, and the
                 complex's sizes, inside size and threshold, counted without
                 building the complex (oracle.lattice_vd_counts; the complex,
                 about 4.2e9 cells, does not fit in this host's memory).

For torus64 and the sphere unions the reference's OWN compiled thinning and
remainingCC (oracle/_ref, built from the reference tree) are also run on the
oracle's complex, and their surviving flags and remaining arrays must equal
the oracle's before anything is written: at these sizes the digests are the
reference's output, not only the restatement's.  The 512^3 complex (4.6e8
cells) is beyond the reference's memory on this host, so that one rests on
the restatement, which the other tests pin to the reference on smaller
complexes.

Run:  python tests/golden/make_fullsize_digests.py [name ...]
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from voxel_ma_gb300 import volumes  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fullsize_digests.json")
T = 0.04


def workloads():
    """name -> (generator, run the reference's own thinning too)."""
    return {
        "torus64": (lambda: volumes.torus_mesh(64), True),
        "spheres256_s0": (lambda: volumes.spheres(256, count=32, seed=0), True),
        "spheres256_s1": (lambda: volumes.spheres(256, count=32, seed=1), True),
        "spheres256_s2": (lambda: volumes.spheres(256, count=32, seed=2), True),
        "grf512": (lambda: volumes.grf(512, sigma=6.0, seed=0), False),
        # sites, feature transform and the complex's sizes only: its complex
        # (about 4.2e9 cells) does not fit in this host's memory
        "grf1024": (lambda: volumes.grf(1024, sigma=6.0, seed=0), False),
    }

FT_ONLY = {"grf1024"}


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def flags01(a) -> np.ndarray:
    return (np.asarray(a) != 0).astype(np.uint8)


def run_ft_case(name: str, gen) -> dict:
    t0 = time.time()
    occ = np.ascontiguousarray(gen())
    xyz, li = oracle.extract_sites(occ)
    d2, ids = oracle.ft(occ.shape, li, threads=os.cpu_count() or 1)
    out = {"shape": list(occ.shape), "stages": "sites+ft+sizes", "occupancy_sha256": volumes.occupancy_sha256(occ),
           "n_sites": int(len(xyz)), "sites": digest(xyz), "ft": digest(d2, ids)}
    del d2, xyz, li
    cnt = oracle.lattice_vd_counts(occ, ids)
    out.update({"t": T, "vd_sizes": [cnt["nv"], cnt["ne"], cnt["nt"]], "inside_size": cnt["inside_size"],
                "thresh": float(np.float32(np.float64(cnt["inside_size"]) * T)),
                "oracle_seconds": round(time.time() - t0, 1)})
    print(name, json.dumps(out), flush=True)
    return out


def run_case(name: str, gen, with_ref: bool) -> dict:
    if name in FT_ONLY:
        return run_ft_case(name, gen)
    t0 = time.time()
    occ = np.ascontiguousarray(gen())
    r = oracle.run_plain(occ, T, threads=os.cpu_count() or 1)
    vd, th = r["vd"], r["thin"]
    rv, re_, rt = r["rem_vts"], r["rem_edges"], r["rem_tris"]
    eu = oracle.euler(len(rv), re_, rt)
    out = {
        "shape": list(occ.shape), "t": T,
        "occupancy_sha256": volumes.occupancy_sha256(occ),
        "n_sites": int(len(r["sites"])), "sites": digest(r["sites"]),
        "ft": digest(r["d2"], r["ids"]),
        "vd_sizes": [int(len(vd["vts"])), int(len(vd["edges"])), int(len(vd["tris"]))],
        "inside_size": float(vd["inside_size"]),
        "complex": digest(vd["vts"], vd["edges"], vd["tris"], vd["em"], vd["fm"]),
        "finalized_edges": int(len(r["fin"]["edges"])),
        "thresh": float(r["thresh"]),
        "thin_stats": th["stats"],
        "keep_v": digest(flags01(th["keep_v"])), "keep_e": digest(flags01(th["keep_e"])),
        "keep_f": digest(flags01(th["keep_f"])), "removed_e": digest(flags01(th["removed_e"])),
        "remaining_sizes": [int(len(rv)), int(len(re_)), int(len(rt))],
        "remaining": digest(rv, re_, rt),
        "remaining_euler": eu,
        "reference_thin": False,
    }
    if with_ref:
        rc = oracle.RefComplex(vd["vts"], vd["edges"], vd["tris"])
        assert np.array_equal(rc.edges(), r["fin"]["edges"]), name
        em_fin = np.zeros(rc.ne, np.float32)
        em_fin[: len(vd["em"])] = vd["em"]
        ref = rc.thin(vd["vm"], em_fin, vd["fm"], r["thresh"], r["thresh"])
        for k in ("keep_v", "keep_e", "keep_f", "removed_e"):
            assert np.array_equal(flags01(ref[k]), flags01(th[k])), (name, k)
        rrv, rre, rrt = rc.remaining()
        assert np.array_equal(rrv, rv) and np.array_equal(rre, re_) and np.array_equal(rrt, rt), name
        assert oracle.ref_euler(rrv, rre, rrt) == eu, name
        out["reference_thin"] = True
        del rc
    out["oracle_seconds"] = round(time.time() - t0, 1)
    print(name, json.dumps(out), flush=True)
    return out


def main(names):
    oracle.build(reference=True, tree=os.environ.get("VOXEL_MA_REFERENCE", "/root/reference"))
    have = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for name, (gen, with_ref) in workloads().items():
        if names and name not in names:
            continue
        if with_ref and not oracle.ref_available():
            raise SystemExit("the reference library (oracle/_ref) is needed: run where the reference tree is")
        have[name] = run_case(name, gen, with_ref)
        with open(OUT, "w") as f:
            json.dump(have, f, indent=1, sort_keys=True)
            f.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main(sys.argv[1:])
