"""Writes .mrc test files (the public MRC2014 layout) from a value volume
indexed (x, y, z), in any mode, axis order and byte order."""
from __future__ import annotations

import numpy as np

MODES = {0: "i1", 1: "i2", 2: "f4", 6: "u2", 12: "f2"}


def write_mrc(vals_xyz: np.ndarray, mode: int = 2, axes=(1, 2, 3), big: bool = False, extended: int = 0,
              stamp: bool = True) -> bytes:
    """axes = the volume axes (1 = x, 2 = y, 3 = z) of columns, rows and
    sections; `extended` bytes of extended header follow the 1024."""
    e = ">" if big else "<"
    dims = vals_xyz.shape
    n = [dims[a - 1] for a in axes]  # columns, rows, sections
    # file array (sections, rows, columns): its axis k runs along volume axis axes[2 - k] - 1
    arr = np.transpose(vals_xyz, [axes[2] - 1, axes[1] - 1, axes[0] - 1])
    h = np.zeros(256, e + "i4")
    h[0:3] = n
    h[3] = mode
    h[7:10] = n
    h[16:19] = axes
    h[23] = extended
    hb = bytearray(h.tobytes())
    hb[40:52] = np.array([float(x) for x in n], e + "f4").tobytes()  # cell lengths
    hb[208:212] = b"MAP "
    if stamp:
        hb[212:216] = bytes([0x11, 0x11, 0, 0]) if big else bytes([0x44, 0x44, 0, 0])
    body = np.ascontiguousarray(arr).astype(np.dtype(MODES[mode]).newbyteorder(e)).tobytes()
    return bytes(hb) + bytes(extended) + body


def value_volume(occ: np.ndarray, mode: int, seed: int = 0) -> np.ndarray:
    """Values whose sign gives occ: positive inside, zero or negative outside
    (unsigned modes: zero outside)."""
    rng = np.random.default_rng(seed)
    mag = rng.integers(1, 100, occ.shape)
    if mode in (6,):
        return np.where(occ > 0, mag, 0).astype(np.uint16)
    neg = -mag * (rng.uniform(size=occ.shape) < 0.7)
    v = np.where(occ > 0, mag, neg)
    if mode in (2, 12):
        v = v.astype(np.float64) * rng.uniform(0.01, 3.0, occ.shape)
        v = np.where(occ > 0, np.maximum(v, 0.01), v)
    return v
