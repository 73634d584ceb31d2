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
* ``grf``         white noise (integer, zero mean) blurred by a periodic
  Gaussian of sigma = 6 voxels, thresholded at 0; exact integer arithmetic,
  so the same field on every host and device.
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


def _grf_weights(sigma: float) -> np.ndarray:
    """Integer taps w_k = round(1024 exp(-k^2 / (2 sigma^2))), k = 0..K, K the
    last k whose tap is at least 1 (sigma = 6: K = 23, taps sum to 15,397)."""
    w = []
    k = 0
    while True:
        v = int(math.floor(1024.0 * math.exp(-k * k / (2.0 * sigma * sigma)) + 0.5))
        if v < 1:
            break
        w.append(v)
        k += 1
    return np.array(w, np.int64)


_SPLITMIX_GAMMA = 0x9E3779B97F4A7C15
_SEED_MUL = 0xD1B54A32D192ED03


def grf_noise(shape, seed: int = 0) -> np.ndarray:
    """White noise of the GRF: int16, in [-510, 510], a pure function of (seed,
    linear voxel index) -- the sum of the four low bytes of splitmix64(index)
    minus 510 (Irwin-Hall of four uniform bytes: mean 0, sd 147.8)."""
    n = int(np.prod(shape))
    out = np.empty(n, np.int16)
    base = np.array([((seed + 1) * _SEED_MUL) & 0xFFFFFFFFFFFFFFFF], np.uint64)
    g = np.uint64(_SPLITMIX_GAMMA)
    m1, m2 = np.uint64(0xBF58476D1CE4E5B9), np.uint64(0x94D049BB133111EB)
    s30, s27, s31, b = np.uint64(30), np.uint64(27), np.uint64(31), np.uint64(255)
    step = 1 << 23
    for a in range(0, n, step):
        z = np.arange(a, min(n, a + step), dtype=np.uint64) * g + base
        z ^= z >> s30
        z *= m1
        z ^= z >> s27
        z *= m2
        z ^= z >> s31
        s = (z & b) + ((z >> np.uint64(8)) & b) + ((z >> np.uint64(16)) & b) + ((z >> np.uint64(24)) & b)
        out[a:a + len(s)] = s.astype(np.int16) - 510
    return out.reshape(shape)


def _blur_exact_numpy(x: np.ndarray, w: np.ndarray) -> np.ndarray:
    """Periodic separable correlation with the symmetric taps w (float64 in and
    out, integer values)."""
    from scipy import ndimage
    taps = np.concatenate([w[:0:-1], w]).astype(np.float64)
    K = len(w) - 1
    for axis in range(3):
        n = x.shape[axis]
        xp = np.take(x, np.arange(-K, n + K) % n, axis=axis)
        y = ndimage.correlate1d(xp, taps, axis=axis, mode="constant", cval=0.0)
        del xp
        sl = [slice(None)] * 3
        sl[axis] = slice(K, K + n)
        x = np.ascontiguousarray(y[tuple(sl)])
        del y
    return x


def _blur_exact_torch(x, w: np.ndarray):
    import torch
    K = len(w) - 1
    for axis in range(3):
        acc = x * float(w[0])
        for k in range(1, K + 1):
            acc += float(w[k]) * (torch.roll(x, k, axis) + torch.roll(x, -k, axis))
        x = acc
    return x


def grf(n: int = 512, sigma: float = 6.0, seed: int = 0, device=None) -> np.ndarray:
    """Thresholded smoothed random field: ``grf_noise`` correlated periodically
    along x, y and z with the integer Gaussian taps of ``sigma``, inside where
    the result is > 0.

    Every partial sum is an integer below 2^53 (|noise| <= 510, taps summing
    to S, 510 S^3 < 2^53), so float64 arithmetic is exact in any summation
    order: the numpy path (host) and the torch path (``device``, any torch
    device) give the same field bit for bit on every machine."""
    w = _grf_weights(sigma)
    S = int(w[0] + 2 * w[1:].sum())
    if 510 * S ** 3 >= 1 << 53:
        raise ValueError(f"sigma {sigma} too large for the exact integer blur")
    noise = grf_noise((n, n, n), seed)
    if device is not None:
        import torch
        x = torch.from_numpy(noise).to(device=device, dtype=torch.float64)
        x = _blur_exact_torch(x, w)
        return (x > 0).to(torch.uint8).cpu().numpy()
    x = _blur_exact_numpy(noise.astype(np.float64), w)
    return (x > 0).astype(np.uint8)


# occupancy_sha256 of the benchmark's volumes, fixed by the generators above
WORKLOAD_SHA256 = {
    "grf512_sigma6_level0": "3837844dac47b0cf6cd54c61271dd70216d12ecd3ceec9ae90c7f9aabb0e94b0",
}


def occupancy_sha256(occ) -> str:
    """sha256 of a volume's shape (3 little-endian int64) and its voxels as
    bytes 0/1, z fastest."""
    import hashlib
    a = np.ascontiguousarray(np.asarray(occ) > 0, dtype=np.uint8)
    h = hashlib.sha256(np.array(a.shape, "<i8").tobytes())
    h.update(a.tobytes())
    return h.hexdigest()


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
