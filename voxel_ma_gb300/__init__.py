"""GB300-native (sm_103a) Voxel Cores hot path: boundary sites, exact feature
transform, lattice Voronoi complex with lambda measures, FIFO-exact thinning
and the remaining complex, behind the C ABI in include/voxelcore_gb300.h."""
from . import volumes  # noqa: F401
from ._lib import VoxelCoreError, load  # noqa: F401

__all__ = ["load", "VoxelCoreError", "volumes"]
