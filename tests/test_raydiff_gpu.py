"""Differentiable raycast: GPU forward loss against the FP64 oracle, and the
hand-written adjoint (pose se(3) and voxel TSDF gradients) against FP64
central finite differences (h = 1e-4 on the pose twist, 1e-3 m on voxels)."""
import numpy as np
import pytest
import torch

import oracle
from superscanner_gb300 import GPUVoxelGrid, synth
from superscanner_gb300.raydiff import raycast_loss, raycast_loss_grad, se3_exp

pytestmark = pytest.mark.gpu

INTR = (525.0, 525.0, 319.5, 239.5)
VL, TRUNC = 0.004, 0.016


def setup(storage="f32"):
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(8, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    g = GPUVoxelGrid(int(1e9), TRUNC, VL, 480, 640, storage=storage, with_color=False, hash_buckets=1 << 18,
                     max_weight=255)
    g.setIntrinsic(*INTR)
    for k in range(8):
        g.integrate_fast(dev[k], P[k].astype(np.float32))
    g.sync()
    d = g.export_blocks(with_color=False)
    o = oracle.MethodGrid64(VL, TRUNC, 480, 640, INTR, 255)
    o.import_blocks(d["coords"], d["sdf"], d["w"])
    return g, o, d, P, depth, dev


def test_forward_loss_matches_fp64():
    g, o, d, P, depth, dev = setup()
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003]) @ P[7]
    L, nv = raycast_loss(g, T, dev[7])
    L64, nv64 = o.raycast_loss(T, depth[7])
    print("loss gpu", L, nv, "fp64", L64, nv64)
    assert nv > 100000 and abs(nv - nv64) <= 1e-3 * nv64
    assert abs(L - L64) <= 1e-3 * L64


def test_adjoint_matches_fp64_finite_differences():
    g, o, d, P, depth, dev = setup()
    T = se3_exp([0.004, -0.003, 0.002, 0.006, -0.004, 0.003]) @ P[7]
    B = g.params.hash_buckets
    gv = torch.zeros((B, 512), dtype=torch.float32, device="cuda")
    L, grad, nv = raycast_loss_grad(g, T, dev[7], grad_voxels=gv)
    h = 1e-4
    fd = np.zeros(6)
    for i in range(6):
        e = np.zeros(6)
        e[i] = h
        fd[i] = (o.raycast_loss(se3_exp(e) @ T, depth[7])[0] - o.raycast_loss(se3_exp(-e) @ T, depth[7])[0]) / (2 * h)
    print("pose grad gpu", grad, "\n          fd ", fd)
    scale = np.abs(fd).max()
    assert np.abs(grad - fd).max() <= 0.05 * scale
    # voxel gradients: the 8 voxels with the largest |dL/ds|
    gvn = gv.cpu().numpy()
    buckets = g.export_buckets()
    q_of = {int(b): q for q, b in enumerate(buckets)}
    flat = np.argsort(-np.abs(gvn).ravel())[:8]
    hv = 1e-3
    rel = []
    for f in flat:
        b, v = divmod(int(f), 512)
        c = d["coords"][q_of[b]]
        assert o.add_voxel(c, v, hv)
        lp = o.raycast_loss(T, depth[7])[0]
        o.add_voxel(c, v, -2 * hv)
        lm = o.raycast_loss(T, depth[7])[0]
        o.add_voxel(c, v, hv)
        fdv = (lp - lm) / (2 * hv)
        print("voxel", b, v, "gpu", gvn[b, v], "fd", fdv)
        rel.append(abs(gvn[b, v] - fdv) / max(abs(fdv), 1e-12))
    assert np.median(rel) < 0.05
