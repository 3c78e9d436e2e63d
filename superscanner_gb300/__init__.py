"""GB300-native SuperScanner reconstruction hot path.

The compute path is ``libss.so`` (hand-written CUDA for sm_103a behind the
C-ABI of ``include/ss_abi.h``). This package mirrors the reference's
operator interface on top of it:

* :class:`GPUVoxelGrid` — ``GPUVoxelGrid`` of src/VoxelGrid/GPUVoxelGrid.h
  (integrate, deIntegrate, raycast, setIntrinsic, cleanMemory).
* :func:`kokkos_icp` — ``kokkosICP`` of src/postprocessing/kokkosICP.h.

There is no CPU fallback: importing the package loads the native library and
raises if it is missing.
"""
from ._native import lib, SSError, check  # noqa: F401
from .voxel_grid import GPUVoxelGrid, depth_to_pcd, normals_from_pcd  # noqa: F401
from .icp import kokkos_icp, PointToPoint, PointToPlane  # noqa: F401
