"""Differentiable raycast over libss.so: the depth / point-to-plane loss of the
rendered model view against an observed depth image, and its adjoint with
respect to the camera pose (se(3), left increment) and the voxel TSDF values."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._native import check, f64x16, lib
from .voxel_grid import GPUVoxelGrid, _dev_ptr, _stream_ptr


def raycast_loss(grid: GPUVoxelGrid, T, depth_obs, lambda_n: float = 1.0, r_max: float = 0.05,
                 max_steps: int = 128, depth_out: torch.Tensor | None = None, stream=None):
    """(loss, valid pixels) of the model view at pose T against depth_obs (CUDA, u16 mm)."""
    loss = C.c_double()
    valid = C.c_int64()
    d = _dev_ptr(depth_obs, 2, (grid.resi, grid.resj), "depth_obs")
    out = C.c_void_p(depth_out.data_ptr()) if depth_out is not None else C.c_void_p()
    check(lib.ss_raycast_loss(grid.handle, f64x16(T), d, float(lambda_n), float(r_max), int(max_steps),
                              C.byref(loss), C.byref(valid), out, _stream_ptr(stream)), "raycast_loss")
    return loss.value, valid.value


def raycast_loss_grad(grid: GPUVoxelGrid, T, depth_obs, lambda_n: float = 1.0, r_max: float = 0.05,
                      max_steps: int = 128, grad_voxels: torch.Tensor | None = None, stream=None):
    """(loss, dL/dxi [6] = (omega, upsilon), valid pixels); grad_voxels ([buckets, 512] float32 CUDA,
    zeroed by the caller) accumulates dL/d(voxel TSDF value)."""
    loss = C.c_double()
    valid = C.c_int64()
    grad = (C.c_double * 6)()
    d = _dev_ptr(depth_obs, 2, (grid.resi, grid.resj), "depth_obs")
    gv = C.c_void_p(grad_voxels.data_ptr()) if grad_voxels is not None else C.c_void_p()
    check(lib.ss_raycast_loss_grad(grid.handle, f64x16(T), d, float(lambda_n), float(r_max), int(max_steps),
                                   C.byref(loss), grad, gv, C.byref(valid), _stream_ptr(stream)),
          "raycast_loss_grad")
    return loss.value, np.array(grad[:]), valid.value


def se3_exp(xi) -> np.ndarray:
    """exp of a twist (omega, upsilon) as a 4x4 matrix (left increment)."""
    w, v = np.asarray(xi[:3], float), np.asarray(xi[3:], float)
    th = np.linalg.norm(w)
    K = np.array([[0, -w[2], w[1]], [w[2], 0, -w[0]], [-w[1], w[0], 0]])
    if th < 1e-12:
        R, V = np.eye(3) + K, np.eye(3) + 0.5 * K
    else:
        A, B, Cc = np.sin(th) / th, (1 - np.cos(th)) / th ** 2, (th - np.sin(th)) / th ** 3
        R = np.eye(3) + A * K + B * K @ K
        V = np.eye(3) + B * K + Cc * K @ K
    T = np.eye(4)
    T[:3, :3], T[:3, 3] = R, V @ v
    return T
