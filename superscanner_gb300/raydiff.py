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


def raycast_loss_grad_masked(grid: GPUVoxelGrid, T, depth_obs, pixel_mask, lambda_n: float = 1.0,
                             r_max: float = 0.05, max_steps: int = 128, stream=None):
    """raycast_loss_grad over the pixels whose pixel_mask (CUDA uint8 [rows, cols]) is non-zero."""
    loss = C.c_double()
    valid = C.c_int64()
    grad = (C.c_double * 6)()
    d = _dev_ptr(depth_obs, 2, (grid.resi, grid.resj), "depth_obs")
    m = _dev_ptr(pixel_mask, 1, (grid.resi, grid.resj), "pixel_mask")
    check(lib.ss_raycast_loss_grad_masked(grid.handle, f64x16(T), d, m, float(lambda_n), float(r_max),
                                          int(max_steps), C.byref(loss), grad, C.c_void_p(), C.byref(valid),
                                          _stream_ptr(stream)), "raycast_loss_grad_masked")
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


def refine_pose(grid: GPUVoxelGrid, T0, depth_obs, *, iters: int = 60, lambda_n: float = 1.0,
                r_max=(0.2, 0.1, 0.05), max_steps: int = 128, step0: float = 1e-3, tol: float = 1e-7, stream=None):
    """Gradient-based refinement of a camera pose (camera -> world) against the
    volume: BFGS on left se(3) increments with a backtracking (Armijo) line
    search, the loss and its pose gradient from the raycast adjoint at every
    evaluation (the march is recomputed, no march state is stored). The first
    step has length step0 along the negative gradient. r_max may be a sequence
    (coarse to fine residual gates): one BFGS run of up to `iters` iterations
    per gate, each starting where the previous one ended. On the synthetic
    room (4 mm FP16 volume, 640x480) the default gates 0.2 / 0.1 / 0.05 m
    brought 20 of 20 starts perturbed by up to 3 deg / 4 cm to within 0.2 mm /
    0.01 deg; a single 0.1 m gate left 6 of them stalled.

    Returns (T, info) with info = {"loss0", "loss", "iters", "evals"}: the
    loss at the start of the first gate and at the end of the last."""
    gates = list(r_max) if np.ndim(r_max) else [float(r_max)]
    T = np.asarray(T0, np.float64).copy()
    info = {"iters": 0, "evals": 0}
    for k, gate in enumerate(gates):
        T, part = _bfgs_pose(grid, T, depth_obs, iters, lambda_n, float(gate), max_steps, step0, tol, stream)
        if k == 0:
            info["loss0"] = part["loss0"]
        info["loss"] = part["loss"]
        info["iters"] += part["iters"]
        info["evals"] += part["evals"]
    return T, info


def _bfgs_pose(grid, T0, depth_obs, iters, lambda_n, r_max, max_steps, step0, tol, stream):
    # The objective is the loss itself (its gradient is exact between gate
    # events). A step must lower it (Armijo) without dropping more than 5 % of
    # the valid pixels: the loss of a view that sees less of the model is
    # smaller, and a search without that guard can walk the camera off the
    # model. Where a BFGS direction finds no step, the scaled negative
    # gradient gets one more try before the run ends.
    def evaluate(T_):
        return raycast_loss_grad(grid, T_, depth_obs, lambda_n, r_max, max_steps, stream=stream)

    T = np.asarray(T0, np.float64).copy()
    L, g, nv = evaluate(T)
    info = {"loss0": L, "iters": 0, "evals": 1}
    if not np.isfinite(L) or float(np.linalg.norm(g)) == 0.0:
        info["loss"] = L
        return T, info

    def scaled_gradient_h(g_):
        return np.eye(6) * (step0 / max(float(np.linalg.norm(g_)), 1e-30))

    H = scaled_gradient_h(g)  # inverse Hessian estimate
    fresh = True
    for it in range(iters):
        p = -H @ g
        slope = float(g @ p)
        if slope >= 0.0:
            H, fresh = scaled_gradient_h(g), True
            p = -H @ g
            slope = float(g @ p)
        a, accepted = 1.0, False
        while a > 1e-6:
            Tn = se3_exp(a * p) @ T
            Ln, gn_vec, nvn = evaluate(Tn)
            info["evals"] += 1
            if np.isfinite(Ln) and Ln <= L + 1e-4 * a * slope and nvn >= 0.95 * nv:
                accepted = True
                break
            a *= 0.5
        if not accepted:
            if fresh:
                break
            H, fresh = scaled_gradient_h(g), True
            continue
        s, y = a * p, gn_vec - g
        sy = float(s @ y)
        if sy > 1e-30:  # BFGS update of the inverse Hessian
            rho = 1.0 / sy
            I = np.eye(6)
            H = (I - rho * np.outer(s, y)) @ H @ (I - rho * np.outer(y, s)) + rho * np.outer(s, s)
            fresh = False
        T, L, g, nv = Tn, Ln, gn_vec, nvn
        info["iters"] = it + 1
        if float(np.linalg.norm(s)) < tol:
            break
    info["loss"] = L
    return T, info
