"""Mesh export of the TSDF on the GPU (the reference meshes on the host:
marchingCubesHost, GPUVoxelGrid.cpp:200-251): marching cubes (or marching
tetrahedra) over the observed cells, then vertices welded on the host and
written as PLY."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._native import check, lib
from .voxel_grid import GPUVoxelGrid, _stream_ptr


def extract_triangles(grid: GPUVoxelGrid, stream=None, method: str = "cubes") -> torch.Tensor:
    """Triangle soup as a CUDA tensor [n, 3, 3] (world coordinates; each
    triangle faces from negative to positive TSDF), by marching cubes (the
    cube conventions of the Open3D extraction the reference runs) or by
    marching tetrahedra (method="tetrahedra")."""
    fn = lib.ss_grid_extract_mesh_cubes if method == "cubes" else lib.ss_grid_extract_mesh
    n = C.c_int64()
    check(fn(grid.handle, 0, None, C.byref(n), _stream_ptr(stream)), "extract_mesh")
    cap = n.value
    out = torch.empty((max(cap, 1), 3, 3), dtype=torch.float32, device=grid.device)
    check(fn(grid.handle, cap, C.c_void_p(out.data_ptr()), C.byref(n), _stream_ptr(stream)), "extract_mesh")
    return out[:min(cap, n.value)]


def weld(tris: np.ndarray, tol: float = 1e-6):
    """(vertices [m, 3], faces [n, 3]) of a triangle soup, vertices closer than tol merged."""
    tris = np.asarray(tris, np.float64).reshape(-1, 3)
    keys = np.round(tris / tol).astype(np.int64)
    _, first, inverse = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    return tris[first], inverse.reshape(-1, 3).astype(np.int64)


def write_ply(path, vertices: np.ndarray, faces: np.ndarray) -> None:
    """Binary little-endian PLY with float vertices and int32 triangle indices."""
    v = np.ascontiguousarray(vertices, np.float32)
    f = np.ascontiguousarray(faces, np.int32)
    header = (f"ply\nformat binary_little_endian 1.0\nelement vertex {len(v)}\n"
              "property float x\nproperty float y\nproperty float z\n"
              f"element face {len(f)}\nproperty list uchar int vertex_indices\nend_header\n")
    rec = np.zeros(len(f), dtype=[("n", "u1"), ("i", "<i4", (3,))])
    rec["n"] = 3
    rec["i"] = f
    with open(path, "wb") as fh:
        fh.write(header.encode("ascii"))
        fh.write(v.astype("<f4").tobytes())
        fh.write(rec.tobytes())
