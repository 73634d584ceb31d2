"""Seeded synthetic cell complexes for finalize / thinning parity tests.

Each generator returns (vts float32 [V,3], edges int32 [E,2], tris int32 [T,3]).
They exercise what cellcomplex::finalize and CellComplexThinning::prune are
sensitive to: edges given in arbitrary order, as unsorted pairs and with
repeats; face sides missing from the edge list; isolated edges and vertices;
closed pockets that cannot collapse; and measures with many ties.
"""
from __future__ import annotations

import numpy as np


def grid_surface(nx: int, ny: int, seed: int, drop: float = 0.1, extra_edges: int = 10,
                 shuffle: bool = True, unsorted: float = 0.0, omit: float = 0.0):
    rng = np.random.default_rng(seed)
    vid = np.arange((nx + 1) * (ny + 1)).reshape(nx + 1, ny + 1)
    xs, ys = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="ij")
    vts = np.stack([xs.ravel(), ys.ravel(), rng.integers(0, 3, xs.size)], -1).astype(np.float32)
    tris = []
    for i in range(nx):
        for j in range(ny):
            a, b, c, d = vid[i, j], vid[i + 1, j], vid[i + 1, j + 1], vid[i, j + 1]
            if rng.uniform() < 0.5:
                tris += [(a, b, c), (a, c, d)]
            else:
                tris += [(a, b, d), (b, c, d)]
    tris = np.array(tris, np.int32)
    keep = rng.uniform(size=len(tris)) >= drop
    tris = tris[keep]
    rng.shuffle(tris)
    # random rotation of each triangle's vertex order
    rot = rng.integers(0, 3, len(tris))
    tris = np.stack([np.roll(t, r) for t, r in zip(tris, rot)]).astype(np.int32) if len(tris) else tris
    es = set()
    for t in tris:
        for s in range(3):
            u, v = int(t[s]), int(t[(s + 1) % 3])
            es.add((min(u, v), max(u, v)))
    edges = sorted(es)
    if omit > 0:
        edges = [e for e in edges if rng.uniform() >= omit]
    nv = len(vts)
    for _ in range(extra_edges):  # isolated edges / dangling chains
        u, v = rng.integers(0, nv, 2)
        if u != v:
            edges.append((int(min(u, v)), int(max(u, v))))
    edges = np.array(edges, np.int32).reshape(-1, 2)
    if shuffle:
        rng.shuffle(edges)
    if unsorted > 0:
        flip = rng.uniform(size=len(edges)) < unsorted
        edges[flip] = edges[flip][:, ::-1]
    if len(edges) > 3:  # a few repeated pairs
        edges = np.concatenate([edges, edges[rng.integers(0, len(edges), 3)]])
    return vts, np.ascontiguousarray(edges), np.ascontiguousarray(tris)


def octahedron_shell():
    """A closed surface (a pocket): nothing is collapsible."""
    vts = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32)
    tris = np.array([[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4], [2, 0, 5], [1, 2, 5], [3, 1, 5], [0, 3, 5]],
                    np.int32)
    edges = np.zeros((0, 2), np.int32)
    return vts, edges, tris


def random_measures(ne: int, nt: int, seed: int, levels: int = 4):
    """Measures on a few levels so that threshold comparisons tie often."""
    rng = np.random.default_rng(seed)
    em = rng.integers(0, levels, ne).astype(np.float32)
    fm = rng.integers(0, levels, nt).astype(np.float32)
    vm = np.zeros(0, np.float32)
    return vm, em, fm
