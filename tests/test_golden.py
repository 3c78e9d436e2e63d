"""Golden fixtures of tests/golden/: ref_fusion.npz comes from the reference's
own code (make_ref_golden.py, oracle/_ref), method.npz from the FP64 method
oracle (make_golden.py). The oracle must keep reproducing them, and the GPU
path must match them."""
from pathlib import Path

import numpy as np
import pytest

import oracle

G = Path(__file__).resolve().parent / "golden"


def _ref():
    return np.load(G / "ref_fusion.npz")


def _dense(d, n):
    sdf = np.zeros((n, 512), np.float32)
    w = np.zeros((n, 512), np.float32)
    sdf[d["map_vox_block"], d["map_vox_index"]] = d["map_sdf"]
    w[d["map_vox_block"], d["map_vox_index"]] = d["map_w"]
    return sdf, w


def _ref_sequence(grid_integrate, grid_deintegrate, d):
    P = d["poses"]
    for k in (0, 1):
        grid_integrate(k)
    grid_deintegrate(1)
    grid_integrate(2)
    return P


def test_oracle_reproduces_reference_fixture():
    d = _ref()
    intr = tuple(d["intr"])
    g = oracle.OracleGrid(0.01, 0.03, 60, 80, intr=intr)
    P = _ref_sequence(lambda k: g.integrate(d["depth"][k], d["rgb"][k], d["poses"][k].astype(np.float32)),
                      lambda k: g.deintegrate(d["depth"][k], d["rgb"][k], d["poses"][k].astype(np.float32)), d)
    e = g.export()
    assert np.array_equal(e["keys"], d["map_keys"]) and np.array_equal(e["coords"], d["map_coords"])
    sdf, w = _dense(d, len(d["map_keys"]))
    assert np.array_equal(e["w"], w) and np.array_equal(e["sdf"], sdf)
    pcd, col = g.raycast(P[2].astype(np.float32))
    assert np.array_equal(pcd, d["ray_pcd"]) and np.array_equal(col, d["ray_col"])
    assert np.array_equal(oracle.normals(oracle.depth_to_pcd(d["depth"][0], intr)), d["normals0"])
    for kind in (0, 1):
        T, rmse, _ = oracle.kokkos_icp(d["depth"][0], d["depth"][1], P[0], P[0], kind, intr)
        np.testing.assert_allclose(T, d[f"icp{kind}_T"], atol=1e-12)
        assert rmse == d[f"icp{kind}_rmse"]


def test_fp64_oracle_reproduces_method_fixture():
    m = np.load(G / "method.npz")
    intr = tuple(m["intr"])
    g = oracle.MethodGrid64(0.004, 0.016, 60, 80, intr, 255)
    for k in range(3):
        g.fuse(m["depth"][k], m["poses"][k])
    vmap, nmap, steps = g.raycast(m["poses"][2], 128, 0.2, 10.0)
    np.testing.assert_allclose(vmap, m["vmap"], atol=1e-9)
    np.testing.assert_allclose(nmap, m["nmap"], atol=1e-9)
    T, inl = oracle.track64(m["depth"][2], vmap, nmap, m["poses"][2], m["track_start"], intr, iters=(6, 4, 3))
    np.testing.assert_allclose(T, m["track_T"], atol=1e-9)
    assert inl == int(m["track_inliers"])
    d = np.linalg.inv(m["poses"][2]) @ T
    assert np.linalg.norm(d[:3, 3]) < 1e-3  # the start pose was 1 cm / 0.5 deg off


@pytest.mark.gpu
def test_gpu_matches_reference_fixture():
    import torch
    from superscanner_gb300 import GPUVoxelGrid, kokkos_icp, depth_to_pcd, normals_from_pcd
    d = _ref()
    intr = tuple(d["intr"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.view(np.int16) if a.dtype == np.uint16 else a)).cuda()
    g = GPUVoxelGrid(int(1e8), 0.03, 0.01, 60, 80, hash_buckets=1 << 14)
    g.setIntrinsic(*intr)
    P = _ref_sequence(lambda k: g.integrate(dev(d["rgb"][k]), dev(d["depth"][k]), d["poses"][k].astype(np.float32)),
                      lambda k: g.deIntegrate(dev(d["rgb"][k]), dev(d["depth"][k]), d["poses"][k].astype(np.float32)),
                      d)
    g.sync()
    e = g.export_blocks()
    assert np.array_equal(e["keys"], d["map_keys"]) and np.array_equal(e["coords"], d["map_coords"])
    sdf, w = _dense(d, len(d["map_keys"]))
    assert np.array_equal(e["w"], w)
    assert np.abs(e["sdf"] - sdf).max() <= 1e-3 * 0.03
    pcd, col = g.raycast(P[2].astype(np.float32))
    assert np.all(pcd.cpu().numpy() == d["ray_pcd"], axis=-1).mean() >= 0.999
    n = normals_from_pcd(depth_to_pcd(dev(d["depth"][0]), *intr))
    assert np.array_equal(n.cpu().numpy(), d["normals0"])
    for kind in (0, 1):
        T, rmse = kokkos_icp(dev(d["depth"][0]), dev(d["depth"][1]), P[0], P[0], kind, intr)
        assert np.abs(T - d[f"icp{kind}_T"]).max() < 1e-4
        assert rmse == pytest.approx(float(d[f"icp{kind}_rmse"]), rel=1e-3)


@pytest.mark.gpu
def test_gpu_method_matches_fp64_fixture():
    import torch
    from superscanner_gb300 import GPUVoxelGrid
    from superscanner_gb300.pipeline import raycast_maps
    m = np.load(G / "method.npz")
    intr = tuple(m["intr"])
    for storage in ("f32", "f16"):
        g = GPUVoxelGrid(int(1e8), 0.016, 0.004, 60, 80, storage=storage, with_color=False, hash_buckets=1 << 14,
                         max_weight=255)
        g.setIntrinsic(*intr)
        for k in range(3):
            g.integrate_fast(torch.from_numpy(m["depth"][k].view(np.int16)).cuda(), m["poses"][k].astype(np.float32))
        v, _ = raycast_maps(g, m["poses"][2].astype(np.float32))
        g.sync()
        dg = v[..., 3].cpu().numpy().astype(np.float64)
        d64 = m["vmap"][..., 3]
        both = (dg > 0) & (d64 > 0)
        assert ((dg > 0) == (d64 > 0)).mean() > 0.98
        assert np.percentile(np.abs(dg[both] - d64[both]), 99) < 1e-3
