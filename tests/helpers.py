"""Shared helpers for the parity tests (CPU oracle side)."""
from __future__ import annotations

import hashlib

import numpy as np


def golden_volume(g, name):
    shape = tuple(int(x) for x in g[f"shape_{name}"])
    n = int(np.prod(shape))
    return np.unpackbits(g[f"vol_{name}"])[:n].reshape(shape).astype(np.uint8)


def golden_flags(g, key, n):
    return np.unpackbits(g[key])[:n].astype(np.uint8)


def golden_volume_names(g):
    return sorted(k[len("vol_"):] for k in g if k.startswith("vol_"))


def golden_cc_names(g):
    return sorted({k.split("_")[1] + "_" + k.split("_")[2] if k.startswith("cc_grid") else k.split("_")[1]
                   for k in g if k.startswith("cc_") and k.endswith("_vts")})


def complex_hash(vts, edges, tris, em, fm) -> bytes:
    h = hashlib.sha256()
    for a in (vts, edges, tris, em, fm):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.digest()


def rem_hash(rv, re_, rt) -> bytes:
    return hashlib.sha256(np.ascontiguousarray(rv).tobytes() + np.ascontiguousarray(re_).tobytes() +
                          np.ascontiguousarray(rt).tobytes()).digest()


def lattice_case(oracle, occ):
    """Oracle sites -> FT -> lattice VD -> finalize (the CPU path up to thinning)."""
    xyz, li = oracle.extract_sites(occ)
    d2, ids = oracle.ft(occ.shape, li)
    vd = oracle.lattice_vd(occ, ids, xyz)
    fin = oracle.finalize(len(vd["vts"]), vd["edges"], vd["tris"])
    em_fin = np.zeros(len(fin["edges"]), np.float32)
    em_fin[: len(vd["em"])] = vd["em"]
    return dict(xyz=xyz, li=li, d2=d2, ids=ids, vd=vd, fin=fin, em_fin=em_fin)
