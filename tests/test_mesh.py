"""Mesh extraction restated in the FP64 oracle (marching cubes and marching
tetrahedra over the observed cells): exact on a linear TSDF, consistently
oriented, closed between cells (no cracks); marching cubes puts one vertex on
each sign-changing edge between voxel centres and closes a sphere."""
import numpy as np
import pytest

import oracle
from superscanner_gb300.mesh import weld

VL, TRUNC = 0.004, 0.016


def plane_grid():
    # sdf of the plane z = 1 + 0.1 x (positive towards -z), observed everywhere in a slab of blocks
    B = 8 * VL
    bs = np.arange(-4, 4)
    coords = np.array([(x, y, z) for x in bs for y in bs for z in range(29, 34)], np.int32)
    k = np.arange(512)
    vl = float(np.float32(VL))  # the grid places voxel centres with its float voxel length
    X = (coords[:, 0:1] * 8 + k % 8 + 0.5) * vl
    Z = (coords[:, 2:3] * 8 + k // 64 + 0.5) * vl
    sdf = np.clip((1.0 + 0.1 * X - Z) / np.sqrt(1.01), -TRUNC, TRUNC)
    g = oracle.MethodGrid64(VL, TRUNC, 480, 640)
    g.import_blocks(coords, sdf.astype(np.float32), np.ones_like(sdf, np.float32))
    return g, bs


@pytest.mark.parametrize("method", ["cubes", "tetrahedra"])
def test_plane_mesh_is_exact_oriented_and_closed(method):
    g, bs = plane_grid()
    tris = g.extract_mesh(method)
    assert len(tris) > 1000
    v = tris.reshape(-1, 3)
    # the interpolated vertices lie on the plane (the float32 sdf values limit this to ~1e-9 m)
    assert np.abs((1.0 + 0.1 * v[:, 0] - v[:, 2]) / np.sqrt(1.01)).max() < 1e-8
    # every triangle faces +sdf, i.e. away from the plane's inside (+z side)
    n = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    assert (n[:, 2] < 0).all()
    # closed: after welding each edge is shared by two triangles, except at the slab's side faces
    V, F = weld(tris)
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    uniq, cnt = np.unique(e, axis=0, return_counts=True)
    assert set(np.unique(cnt)) <= {1, 2}
    mid = (V[uniq[cnt == 1, 0]] + V[uniq[cnt == 1, 1]]) / 2
    vl = float(np.float32(VL))
    lo, hi = (bs[0] * 8 + 0.5) * vl, ((bs[-1] + 1) * 8 - 0.5) * vl
    on_side = (np.abs(mid[:, 0] - lo) < 1e-9) | (np.abs(mid[:, 0] - hi) < 1e-9) | \
              (np.abs(mid[:, 1] - lo) < 1e-9) | (np.abs(mid[:, 1] - hi) < 1e-9)
    assert on_side.all()


def test_marching_cubes_closes_a_sphere_with_vertices_on_grid_edges():
    vl = float(np.float32(VL))
    r, c0 = 0.05, np.array([0.013, -0.007, 0.021])
    bs = np.arange(-3, 3)
    coords = np.array([(x, y, z) for x in bs for y in bs for z in bs], np.int32)
    k = np.arange(512)
    P = np.stack([(coords[:, a:a + 1] * 8 + (k // (8 ** a)) % 8 + 0.5) * vl for a in range(3)], axis=-1)
    sdf = np.clip(np.linalg.norm(P - c0, axis=-1) - r, -TRUNC, TRUNC)
    g = oracle.MethodGrid64(VL, TRUNC, 480, 640)
    g.import_blocks(coords, sdf.astype(np.float32), np.ones_like(sdf, np.float32))
    tris = g.extract_mesh("cubes")
    V, F = weld(tris)
    # closed and consistently oriented: every directed edge once, its reverse once
    d = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    key = d[:, 0] * len(V) + d[:, 1]
    rev = d[:, 1] * len(V) + d[:, 0]
    assert len(np.unique(key)) == len(key)
    assert np.array_equal(np.sort(key), np.sort(rev))
    assert len(V) - len(key) // 2 + len(F) == 2  # Euler characteristic of a sphere
    # outward: enclosed volume positive and close to the sphere's
    vol = np.einsum("ij,ij->i", V[F[:, 0]], np.cross(V[F[:, 1]], V[F[:, 2]])).sum() / 6
    assert abs(vol / (4 / 3 * np.pi * r ** 3) - 1) < 0.01
    # each vertex lies on a grid edge: two of its coordinates are voxel-centre coordinates
    on = np.abs((V / vl - 0.5) - np.round(V / vl - 0.5)) < 1e-6
    assert (on.sum(axis=1) >= 2).all()
    # near the sphere (linear interpolation of a curved field)
    assert np.abs(np.linalg.norm(V - c0, axis=1) - r).max() < 0.1 * vl
