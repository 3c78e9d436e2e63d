"""Mesh extraction restated in the FP64 oracle (marching tetrahedra over the
observed cells): exact on a linear TSDF, consistently oriented, closed
between cells (no cracks)."""
import numpy as np

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


def test_plane_mesh_is_exact_oriented_and_closed():
    g, bs = plane_grid()
    tris = g.extract_mesh()
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
