"""vc_write_remaining on the GPU path's remaining complex: the .ply, .r and
.ma files equal, byte for byte, the oracle's writers fed with the oracle's
own remaining complex, radii and .ma edge list."""
import numpy as np
import pytest

import oracle as O
from voxel_ma_gb300 import _lib, volumes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [5, 6])
def test_write_remaining_matches_the_oracle(gpu_ctx, tmp_path, seed):
    occ = volumes.grf(40, sigma=3.0, seed=seed)
    ref = O.run_plain(occ, t=0.04)
    gpu_ctx.run_plain(occ, 0.04)
    gpu_ctx.write_remaining(str(tmp_path / "gpu"))
    rv, re_, rt = ref["rem_vts"], ref["rem_edges"], ref["rem_tris"]
    radii = ref["vd"]["radius"][ref["thin"]["keep_v"].astype(bool)]
    base = str(tmp_path / "oracle")
    O.write_ply(base + ".ply", rv, re_, rt)
    O.write_radii(base + ".r", rv, radii)
    O.write_dotma(base + ".ma", rv, radii, O.dotma_edges(re_, rt), rt)
    for ext in (".ply", ".r", ".ma"):
        got = open(str(tmp_path / "gpu") + ext, "rb").read()
        assert got == open(base + ext, "rb").read(), ext
    assert len(got) > 1000


def test_write_remaining_needs_the_lattice_complex_for_radii(gpu_ctx, tmp_path):
    # a given complex has no radii: the PLY is written, .r / .ma are refused
    vts = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], np.float32)
    tris = np.array([[0, 1, 2], [1, 3, 2]], np.int32)
    gpu_ctx.set_complex(vts, np.zeros((0, 2), np.int32), tris)
    ne = gpu_ctx.finalize()
    gpu_ctx.set_measures(np.zeros(4, np.float32), np.zeros(ne, np.float32), np.ones(2, np.float32))
    gpu_ctx.thin(0.5, 0.5)
    gpu_ctx.remaining()
    gpu_ctx.write_remaining(str(tmp_path / "given"), ply=True, radii=False, ma=False)
    assert open(str(tmp_path / "given.ply")).read().startswith("ply\n")
    with pytest.raises(_lib.VoxelCoreError) as ei:
        gpu_ctx.write_remaining(str(tmp_path / "given"), ply=False, radii=True, ma=False)
    assert ei.value.status == _lib.VC_ERR_STATE
