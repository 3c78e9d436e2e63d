"""Analytic test scenes shared by the oracle and GPU tests.

wavy_wall: a tilted, sinusoidally curved wall z = h(x, y) in front of a camera
at the origin looking down +z, stored as voxel blocks with the signed distance
(h - z) / |(h_x, h_y, -1)| (positive towards the camera) clipped to the
truncation, weight 1 everywhere. The slab of blocks covers the whole field of
view, so every ray hits the same smooth sheet and the loss of the
differentiable raycast is smooth in the pose: finite differences of it are
clean, unlike on a fused scene where silhouettes and dropout make pixels
switch in and out of the loss.
"""
import numpy as np

VL, TRUNC = 0.004, 0.016


def wall_height(x, y):
    return 1.0 + 0.03 * np.sin(4 * x) * np.cos(3 * y) + 0.1 * x


def wavy_wall(rows=120, cols=160, noise=0.002, seed=1):
    """Returns (coords [n,3] int32, sdf [n,512] f32, w [n,512] f32, obs [rows,cols] u16 mm, intr)."""
    f = 131.25 * cols / 160
    intr = (f, f, (cols - 1) / 2, (rows - 1) / 2)
    half_x = (cols / 2) / f * 1.25 + 0.1
    half_y = (rows / 2) / f * 1.25 + 0.1
    B = 8 * VL
    bxs = np.arange(int(np.floor(-half_x / B)), int(np.ceil(half_x / B)))
    bys = np.arange(int(np.floor(-half_y / B)), int(np.ceil(half_y / B)))
    bzs = np.arange(int(np.floor(0.8 / B)), int(np.ceil(1.25 / B)))
    coords = np.array([(x, y, z) for x in bxs for y in bys for z in bzs], np.int32)
    k = np.arange(512)
    kx, ky, kz = k % 8, (k // 8) % 8, k // 64
    X = (coords[:, 0:1] * 8 + kx + 0.5) * VL
    Y = (coords[:, 1:2] * 8 + ky + 0.5) * VL
    Z = (coords[:, 2:3] * 8 + kz + 0.5) * VL
    hx = 0.12 * np.cos(4 * X) * np.cos(3 * Y) + 0.1
    hy = -0.09 * np.sin(4 * X) * np.sin(3 * Y)
    sdf = np.clip((wall_height(X, Y) - Z) / np.sqrt(1 + hx * hx + hy * hy), -TRUNC, TRUNC).astype(np.float32)
    w = np.ones_like(sdf)
    jj, ii = np.meshgrid(np.arange(cols), np.arange(rows))
    dx = (jj - intr[2]) / intr[0]
    dy = (ii - intr[3]) / intr[1]
    t = np.ones_like(dx)
    for _ in range(60):  # fixed point of t = h(t dx, t dy): depth of the wall along each pixel ray
        t = wall_height(t * dx, t * dy)
    rng = np.random.default_rng(seed)
    obs = np.round((t + rng.normal(0, noise, t.shape)) * 1000).astype(np.uint16)
    return coords, sdf, w, obs, intr
