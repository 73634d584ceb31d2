"""MRC density maps (readMRC, src/importers.cpp:45-60).  Tao Ju's reader,
which the reference calls, is not in its tree: parity with it is unpinned.
Here the oracle's restatement of the public MRC2014 layout reads files
written for known volumes in every mode, axis order and byte order; the GPU
reader (vc_set_volume_mrc) must give the same occupancy and sites."""
import numpy as np
import pytest

import oracle as O
from mrc_files import value_volume, write_mrc
from voxel_ma_gb300 import volumes

CASES = [(mode, axes, big, ext) for mode in (0, 1, 2, 6, 12) for axes, big, ext in
         (((1, 2, 3), False, 0), ((3, 2, 1), True, 0), ((2, 3, 1), False, 160), ((1, 3, 2), False, 0))]


def _occ():
    rng = np.random.default_rng(3)
    return (rng.uniform(size=(13, 21, 17)) < 0.5).astype(np.uint8)


@pytest.mark.parametrize("mode,axes,big,ext", CASES)
def test_oracle_reads_what_was_written(mode, axes, big, ext):
    occ = _occ()
    data = write_mrc(value_volume(occ, mode, seed=mode), mode, axes, big, ext)
    got = O.mrc_decode(data)
    assert got is not None and np.array_equal(got, occ)


def test_unstamped_files_and_malformed_ones():
    occ = _occ()
    for big in (False, True):
        assert np.array_equal(O.mrc_decode(write_mrc(value_volume(occ, 2), 2, big=big, stamp=False)), occ)
    data = write_mrc(value_volume(occ, 2), 2)
    assert O.mrc_decode(data[:-1]) is None          # truncated values
    assert O.mrc_decode(data[:900]) is None         # truncated header
    bad = bytearray(data)
    bad[12:16] = np.array([3], "<i4").tobytes()     # complex mode
    assert O.mrc_decode(bytes(bad)) is None


def test_mrc_dims_without_a_gpu():
    """vc_mrc_dims reads the header on the host."""
    import ctypes
    from voxel_ma_gb300 import _lib
    lib = _lib.load()
    occ = _occ()
    for axes in ((1, 2, 3), (3, 1, 2)):
        data = np.frombuffer(write_mrc(value_volume(occ, 1), 1, axes), np.uint8)
        dims = np.zeros(3, np.int32)
        assert lib.vc_mrc_dims(data.ctypes.data_as(ctypes.c_void_p), len(data),
                               dims.ctypes.data_as(ctypes.c_void_p)) == _lib.VC_OK
        assert tuple(dims) == occ.shape
    short = np.zeros(100, np.uint8)
    assert lib.vc_mrc_dims(short.ctypes.data_as(ctypes.c_void_p), 100,
                           dims.ctypes.data_as(ctypes.c_void_p)) == _lib.VC_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("mode,axes,big,ext", CASES)
def test_gpu_reader_matches_the_oracle(gpu_ctx, mode, axes, big, ext):
    occ = _occ() if mode != 2 else volumes.csg(5, 24, 48)
    data = write_mrc(value_volume(occ, mode, seed=mode), mode, axes, big, ext)
    ref = O.mrc_decode(data)
    shape = gpu_ctx.set_volume_mrc(data)
    assert shape == ref.shape
    assert np.array_equal(gpu_ctx.volume(), ref)
    gpu_ctx.extract_sites()
    xyz, _ = O.extract_sites(ref)
    assert np.array_equal(gpu_ctx.sites(), xyz)


@pytest.mark.gpu
def test_gpu_mrc_rejects_malformed(gpu_ctx):
    from voxel_ma_gb300 import _lib
    data = write_mrc(value_volume(_occ(), 2), 2)
    for bad in (data[:-1], data[:900]):
        with pytest.raises(_lib.VoxelCoreError) as ei:
            gpu_ctx.set_volume_mrc(bad)
        assert ei.value.status == _lib.VC_ERR_ARG
