"""GPU mesh extraction against the FP64 oracle's on the same volume, by
marching cubes and by marching tetrahedra: the same triangles (count,
centroids within 10 um, orientation)."""
import numpy as np
import pytest
import torch

import oracle
from scenes import wavy_wall, VL as WVL, TRUNC as WTRUNC
import synth
from superscanner_gb300 import GPUVoxelGrid
from superscanner_gb300.mesh import extract_triangles

pytestmark = pytest.mark.gpu


def compare(g, vl, trunc, method):
    d = g.export_blocks(with_color=False)
    o = oracle.MethodGrid64(vl, trunc, g.resi, g.resj)
    o.import_blocks(d["coords"], d["sdf"], d["w"])
    t64 = o.extract_mesh(method)
    t32 = extract_triangles(g, method=method).cpu().numpy().astype(np.float64)
    assert len(t32) == len(t64) and len(t32) > 1000
    from scipy.spatial import cKDTree
    c32, c64 = t32.mean(axis=1), t64.mean(axis=1)
    dist, idx = cKDTree(c64).query(c32)
    back, _ = cKDTree(c32).query(c64)
    assert dist.max() < 1e-5 and back.max() < 1e-5
    # zero-area triangles where the surface passes through a voxel centre can share a centroid
    assert len(idx) - len(np.unique(idx)) <= 1e-4 * len(idx)
    n32 = np.cross(t32[:, 1] - t32[:, 0], t32[:, 2] - t32[:, 0])
    n64 = np.cross(t64[idx, 1] - t64[idx, 0], t64[idx, 2] - t64[idx, 0])
    # orientation of non-degenerate triangles (|n| = twice the area; typical cells give ~vl^2 = 1.6e-5 m^2)
    big = np.linalg.norm(n64, axis=1) > 1e-8
    assert (np.sum(n32[big] * n64[big], axis=1) > 0).mean() >= 0.9999
    return len(t32)


@pytest.mark.parametrize("method", ["cubes", "tetrahedra"])
def test_mesh_of_the_analytic_wall(method):
    coords, sdf, w, obs, intr = wavy_wall()
    g = GPUVoxelGrid(int(1e9), WTRUNC, WVL, obs.shape[0], obs.shape[1], storage="f32", with_color=False,
                     hash_buckets=1 << 17)
    g.setIntrinsic(*intr)
    g.import_blocks(coords, sdf, w)
    g.sync()
    compare(g, WVL, WTRUNC, method)


@pytest.mark.parametrize("method", ["cubes", "tetrahedra"])
def test_mesh_of_a_fused_room_f16(method):
    INTR = (525.0, 525.0, 319.5, 239.5)
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(10, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    g = GPUVoxelGrid(int(1e9), 0.016, 0.004, 480, 640, storage="f16", with_color=False, hash_buckets=1 << 18,
                     max_weight=255)
    g.setIntrinsic(*INTR)
    for k in range(10):
        g.integrate_fast(torch.from_numpy(np.ascontiguousarray(depth[k].view(np.int16))).cuda(),
                         P[k].astype(np.float32))
    g.sync()
    n = compare(g, 0.004, 0.016, method)
    assert n > 100000
