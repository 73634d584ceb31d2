"""Allocation-free site extraction (vc_extract_sites_noalloc).

Callers that cannot allocate device memory -- code running under an
allocator or framework that owns the device heap, or a plugin that must not
grow the process's device footprint -- use this entry point: it takes its
scratch from a fixed array inside the library instead of cudaMalloc.  This
test calls it through the C ABI twice in a row (the second call reuses the
scratch the first one left behind) and checks both results against the
context-based entry points, bit for bit (sites are half-integer floats).
It runs last so that a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from voxel_ma_gb300 import _lib, volumes

pytestmark = pytest.mark.gpu

MAX_VOXELS = 1 << 22


def _noalloc(lib, occ_dev, shape, out_dev, capacity):
    n = ctypes.c_int64(-1)
    st = lib.vc_extract_sites_noalloc(ctypes.c_void_p(occ_dev.data_ptr()), shape[0], shape[1], shape[2],
                                      ctypes.c_void_p(out_dev.data_ptr()) if out_dev is not None else None,
                                      capacity, ctypes.byref(n), None)
    return st, n.value


def test_noalloc_sites_match_context_path_twice():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxel_ma_gb300 import api
    lib = _lib.load()
    rng = np.random.default_rng(4)
    cases = [volumes.grf(48, sigma=6.0, seed=2), volumes.torus_mesh(32),
             (rng.uniform(size=(37, 19, 53)) < 0.5).astype(np.uint8), np.ones((1, 1, 1), np.uint8),
             volumes.grf(160, sigma=6.0, seed=5)[:, :, :160]]
    with api.Context(0) as ctx:
        for occ in cases:
            occ = np.ascontiguousarray(occ)
            ctx.set_volume(occ)
            n_ref = ctx.extract_sites()
            ref = ctx.sites()
            occ_dev = torch.from_numpy(occ).cuda()
            out = torch.empty((max(n_ref, 1), 3), dtype=torch.float32, device="cuda")
            for call in range(2):
                out.fill_(float("nan"))
                torch.cuda.synchronize()
                st, n = _noalloc(lib, occ_dev, occ.shape, out, n_ref)
                assert st == _lib.VC_OK, (call, st)
                assert n == n_ref, (call, n, n_ref)
                assert np.array_equal(out[:n].cpu().numpy(), ref), call


def test_noalloc_limits():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    occ = np.ascontiguousarray(volumes.torus_mesh(32))
    occ_dev = torch.from_numpy(occ).cuda()
    # too little room: the count comes back, nothing is written, status VC_ERR_ARG
    out = torch.full((4, 3), -7.0, device="cuda")
    st, n = _noalloc(lib, occ_dev, occ.shape, out, 4)
    assert st == _lib.VC_ERR_ARG and n > 4
    assert bool((out == -7.0).all())
    # a volume beyond the static scratch is rejected before any GPU work
    n = ctypes.c_int64(-1)
    st = lib.vc_extract_sites_noalloc(ctypes.c_void_p(occ_dev.data_ptr()), 256, 256, 65, None, 0, ctypes.byref(n),
                                      None)
    assert 256 * 256 * 65 > MAX_VOXELS and st == _lib.VC_ERR_ARG and n.value == -1
