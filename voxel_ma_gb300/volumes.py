"""Seeded synthetic occupancy volumes for the workloads the hot path is measured on.

All volumes are ``uint8`` arrays of shape (X, Y, Z), x-major with z fastest,
1 = inside.  Voxel (i, j, k) covers [i/n, (i+1)/n] x ... of the unit cube and is
inside when its centre is inside the solid.  These generators stand in for the
reference's .mrc/.sof models, which are not available; the shapes, sizes and
value distributions follow the workload definitions:

* ``torus_mesh``  closed triangle-mesh torus, major radius 0.35, minor 0.15,
  centred in the unit cube, 64 (u) x 32 (v) segments, voxel centre inside by a
  parity ray test; 64^3.
* ``spheres``     union of 32 spheres, centres U[0.2,0.8]^3, radii U[0.05,0.20].
* ``grf``         white noise N(0,1) blurred by a periodic Gaussian of
  sigma = 6 voxels, thresholded at 0.
* ``csg``         random union/difference of 1-8 spheres, boxes and capsules in
  a box whose per-axis sizes are log-uniform in [lo, hi].
"""
from __future__ import annotations

import math

import numpy as np


def _centres(n: int) -> np.ndarray:
    return (np.arange(n, dtype=np.float64) + 0.5) / n


def torus_mesh(n: int = 64, R: float = 0.35, r: float = 0.15, nu: int = 64, nv: int = 32) -> np.ndarray:
    """Voxelize a closed triangle-mesh torus by counting +z ray crossings per column."""
    u = 2 * math.pi * np.arange(nu) / nu
    v = 2 * math.pi * np.arange(nv) / nv
    U, V = np.meshgrid(u, v, indexing="ij")
    P = np.stack([0.5 + (R + r * np.cos(V)) * np.cos(U), 0.5 + (R + r * np.cos(V)) * np.sin(U),
                  0.5 + r * np.sin(V)], -1)  # (nu, nv, 3)
    tris = []
    for i in range(nu):
        for j in range(nv):
            a, b = P[i, j], P[(i + 1) % nu, j]
            c, d = P[(i + 1) % nu, (j + 1) % nv], P[i, (j + 1) % nv]
            tris.append((a, b, c))
            tris.append((a, c, d))
    T = np.array(tris)  # (nt, 3, 3)
    xs = _centres(n)
    X, Y = np.meshgrid(xs, xs, indexing="ij")
    px, py = X.ravel(), Y.ravel()
    hits = [[] for _ in range(n * n)]
    for t in T:
        (x0, y0, z0), (x1, y1, z1), (x2, y2, z2) = t
        det = (y1 - y2) * (x0 - x2) + (x2 - x1) * (y0 - y2)
        if abs(det) < 1e-18:
            continue
        lo_x, hi_x = min(x0, x1, x2), max(x0, x1, x2)
        lo_y, hi_y = min(y0, y1, y2), max(y0, y1, y2)
        m = (px >= lo_x) & (px <= hi_x) & (py >= lo_y) & (py <= hi_y)
        idx = np.nonzero(m)[0]
        if idx.size == 0:
            continue
        qx, qy = px[idx], py[idx]
        w0 = ((y1 - y2) * (qx - x2) + (x2 - x1) * (qy - y2)) / det
        w1 = ((y2 - y0) * (qx - x2) + (x0 - x2) * (qy - y2)) / det
        w2 = 1.0 - w0 - w1
        ok = (w0 >= 0) & (w1 >= 0) & (w2 > 0)  # half-open rule: shared edges counted once
        for q, zz in zip(idx[ok], (w0 * z0 + w1 * z1 + w2 * z2)[ok]):
            hits[q].append(zz)
    occ = np.zeros((n, n, n), np.uint8)
    zs = xs
    for q in range(n * n):
        if not hits[q]:
            continue
        h = np.sort(np.array(hits[q]))
        cnt = np.searchsorted(h, zs)  # crossings below each voxel centre
        occ[q // n, q % n, :] = (cnt % 2).astype(np.uint8)
    return occ


def spheres(n: int = 256, count: int = 32, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    C = rng.uniform(0.2, 0.8, size=(count, 3))
    Rs = rng.uniform(0.05, 0.20, size=count)
    xs = _centres(n)
    occ = np.zeros((n, n, n), bool)
    for c, rad in zip(C, Rs):
        lo = np.searchsorted(xs, c - rad)
        hi = np.searchsorted(xs, c + rad, side="right")
        sx, sy, sz = (slice(int(lo[k]), int(hi[k])) for k in range(3))
        dx = (xs[sx] - c[0])[:, None, None]
        dy = (xs[sy] - c[1])[None, :, None]
        dz = (xs[sz] - c[2])[None, None, :]
        occ[sx, sy, sz] |= dx * dx + dy * dy + dz * dz <= rad * rad
    return occ.astype(np.uint8)


def _gauss_kernel_fft(n: int, sigma: float) -> np.ndarray:
    f = np.fft.fftfreq(n)
    return np.exp(-2.0 * (math.pi * sigma * f) ** 2)


def grf(n: int = 512, sigma: float = 6.0, seed: int = 0, device=None) -> np.ndarray:
    """Thresholded smoothed Gaussian random field.  ``device`` = a torch CUDA device for large n."""
    if device is not None:
        import torch
        g = torch.Generator(device="cpu").manual_seed(seed)
        w = torch.randn((n, n, n), generator=g, dtype=torch.float32).to(device)
        Wf = torch.fft.rfftn(w)
        del w
        f = torch.fft.fftfreq(n, device=device, dtype=torch.float32)
        fr = torch.fft.rfftfreq(n, device=device, dtype=torch.float32)
        kx = torch.exp(-2.0 * (math.pi * sigma * f) ** 2)
        kz = torch.exp(-2.0 * (math.pi * sigma * fr) ** 2)
        Wf *= kx[:, None, None] * kx[None, :, None] * kz[None, None, :]
        out = torch.fft.irfftn(Wf, s=(n, n, n))
        del Wf
        occ = (out > 0).to(torch.uint8).cpu().numpy()
        return occ
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((n, n, n), dtype=np.float32)
    Wf = np.fft.rfftn(w)
    k = _gauss_kernel_fft(n, sigma)
    kz = np.exp(-2.0 * (math.pi * sigma * np.fft.rfftfreq(n)) ** 2)
    Wf *= (k[:, None, None] * k[None, :, None] * kz[None, None, :])
    out = np.fft.irfftn(Wf, s=(n, n, n), axes=(0, 1, 2))
    return (out > 0).astype(np.uint8)


def _csg_plan(seed: int, lo: int, hi: int):
    """Dims and primitive list of one random CSG volume (numpy RNG, seeded)."""
    rng = np.random.default_rng(seed)
    dims = np.exp(rng.uniform(math.log(lo), math.log(hi), size=3)).astype(int)
    dims = np.clip(dims, lo, hi)
    prims = []
    nprim = int(rng.integers(1, 9))
    for p in range(nprim):
        kind = int(rng.integers(0, 3))
        c = rng.uniform(0.25, 0.75, size=3)
        if kind == 0:
            prm = (rng.uniform(0.08, 0.3),)
        elif kind == 1:
            prm = (rng.uniform(0.08, 0.3, size=3),)
        else:
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            ln = rng.uniform(0.1, 0.4)
            rad = rng.uniform(0.05, 0.18)
            prm = (d, ln, rad)
        subtract = p > 0 and rng.uniform() < 0.25
        prims.append((kind, c, prm, subtract))
    return tuple(int(x) for x in dims), prims


def csg(seed: int, lo: int = 32, hi: int = 192, device=None):
    """Random CSG of 1-8 primitives (spheres, boxes, capsules) in a box of log-uniform sizes.

    With ``device`` (a torch CUDA device) the volume is evaluated there and a
    uint8 tensor is returned; the primitives are the same, but capsule
    boundaries may round differently from the numpy evaluation."""
    (X, Y, Z), prims = _csg_plan(seed, lo, hi)
    if device is not None:
        import torch
        ax = [(torch.arange(d, device=device, dtype=torch.float64) + 0.5) / d for d in (X, Y, Z)]
        P = torch.meshgrid(*ax, indexing="ij")
        occ = torch.zeros((X, Y, Z), dtype=torch.bool, device=device)
        for kind, c, prm, subtract in prims:
            if kind == 0:
                m = (P[0] - c[0]) ** 2 + (P[1] - c[1]) ** 2 + (P[2] - c[2]) ** 2 <= prm[0] * prm[0]
            elif kind == 1:
                h = prm[0]
                m = (torch.abs(P[0] - c[0]) <= h[0]) & (torch.abs(P[1] - c[1]) <= h[1]) & \
                    (torch.abs(P[2] - c[2]) <= h[2])
            else:
                d, ln, rad = prm
                a = c - d * ln / 2
                r0, r1, r2 = P[0] - a[0], P[1] - a[1], P[2] - a[2]
                t = torch.clamp(r0 * d[0] + r1 * d[1] + r2 * d[2], 0.0, ln)
                m = (r0 - t * d[0]) ** 2 + (r1 - t * d[1]) ** 2 + (r2 - t * d[2]) ** 2 <= rad * rad
            occ = occ & ~m if subtract else occ | m
        return occ.to(torch.uint8)
    ax = [(np.arange(d) + 0.5) / d for d in (X, Y, Z)]
    P = np.meshgrid(*ax, indexing="ij")
    occ = np.zeros((X, Y, Z), bool)
    for kind, c, prm, subtract in prims:
        if kind == 0:
            m = (P[0] - c[0]) ** 2 + (P[1] - c[1]) ** 2 + (P[2] - c[2]) ** 2 <= prm[0] * prm[0]
        elif kind == 1:
            h = prm[0]
            m = (np.abs(P[0] - c[0]) <= h[0]) & (np.abs(P[1] - c[1]) <= h[1]) & (np.abs(P[2] - c[2]) <= h[2])
        else:
            d, ln, rad = prm
            a = c - d * ln / 2
            rel = np.stack([P[0] - a[0], P[1] - a[1], P[2] - a[2]], -1)
            t = np.clip(rel @ d, 0.0, ln)
            q = rel - t[..., None] * d
            m = (q ** 2).sum(-1) <= rad * rad
        if subtract:
            occ &= ~m
        else:
            occ |= m
    return occ.astype(np.uint8)
