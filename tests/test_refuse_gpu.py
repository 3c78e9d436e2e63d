"""Batched loop-closure re-fusion (ss_refuse_batch) equals the 2n sequential
deintegrate / integrate calls bit for bit, for both storage forms and both
arithmetic variants, with keyframes of uneven coverage (occlusion masks)."""
import numpy as np
import pytest
import torch

import synth
from superscanner_gb300 import GPUVoxelGrid

pytestmark = pytest.mark.gpu

INTR = (525.0, 525.0, 319.5, 239.5)


def delta(rng, deg=2.0, cm=3.0):
    ax = rng.normal(size=3)
    ax /= np.linalg.norm(ax)
    a = np.radians(rng.uniform(0, deg))
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    D = np.eye(4)
    D[:3, :3] = np.eye(3) + np.sin(a) * K + (1 - np.cos(a)) * K @ K
    v = rng.normal(size=3)
    D[:3, 3] = v / np.linalg.norm(v) * rng.uniform(0, cm / 100)
    return D


@pytest.mark.parametrize("storage,exact", [("f32", True), ("f32", False), ("f16", False), ("f16", True)])
def test_batched_refusion_equals_sequential(storage, exact):
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(40, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    masks = synth.occlusion_masks(40, 480, 640, seed=99)
    depth = np.where(masks, depth, 0).astype(np.uint16)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    rng = np.random.default_rng(5)
    kf = list(range(0, 40, 3))
    T_new = np.stack([delta(rng) @ P[k] for k in kf])
    out = []
    for batched in (False, True):
        g = GPUVoxelGrid(int(1e9), 0.016, 0.004, 480, 640, storage=storage, with_color=False,
                         hash_buckets=1 << 18, max_weight=255)
        g.setIntrinsic(*INTR)
        if batched:
            g.refuse_batch([], [], [])  # no keyframes: allocates the batch buffers, changes nothing
        for k in range(40):
            if exact:
                g.integrate(None, dev[k], P[k].astype(np.float32), withColor=False)
            else:
                g.integrate_fast(dev[k], P[k].astype(np.float32))
        if batched:
            g.refuse_batch([dev[k] for k in kf], P[kf], T_new, exact=exact)
        else:
            for q, k in enumerate(kf):
                if exact:
                    g.deIntegrate(None, dev[k], P[k].astype(np.float32), withColor=False)
                    g.integrate(None, dev[k], T_new[q].astype(np.float32), withColor=False)
                else:
                    g.integrate_fast(dev[k], P[k].astype(np.float32), deint=True)
                    g.integrate_fast(dev[k], T_new[q].astype(np.float32))
        g.sync()
        out.append(g.export_blocks(with_color=False))
        g.close()
    a, b = out
    assert np.array_equal(a["keys"], b["keys"]) and np.array_equal(a["coords"], b["coords"])
    assert np.array_equal(a["w"], b["w"])
    assert np.array_equal(a["sdf"], b["sdf"])


def test_batched_refusion_matches_oracle():
    """The exact batched re-fusion against the CPU oracle's sequential
    deIntegrate(old pose) + integrate(new pose) per keyframe (the reference's
    re-fusion, src/core/integrate.cpp:109-113, with reference arithmetic):
    block set, weights and TSDF bit for bit (FP32 storage, no weight cap)."""
    import oracle
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(24, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    masks = synth.occlusion_masks(24, 480, 640, seed=99)
    depth = np.where(masks, depth, 0).astype(np.uint16)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    rng = np.random.default_rng(5)
    kf = list(range(0, 24, 2))
    T_new = np.stack([delta(rng) @ P[k] for k in kf])
    g = GPUVoxelGrid(int(1e9), 0.016, 0.004, 480, 640, storage="f32", with_color=False, hash_buckets=1 << 18)
    g.setIntrinsic(*INTR)
    o = oracle.OracleGrid(0.004, 0.016, 480, 640, intr=INTR)
    for k in range(24):
        g.integrate(None, dev[k], P[k].astype(np.float32), withColor=False)
        o.integrate(depth[k], None, P[k].astype(np.float32), with_color=False)
    g.refuse_batch([dev[k] for k in kf], P[kf], T_new, exact=True)
    for q, k in enumerate(kf):
        o.deintegrate(depth[k], None, P[k].astype(np.float32), with_color=False)
        o.integrate(depth[k], None, T_new[q].astype(np.float32), with_color=False)
    g.sync()
    a, b = g.export_blocks(with_color=False), o.export()
    g.close()
    assert np.array_equal(a["keys"], b["keys"]) and np.array_equal(a["coords"], b["coords"])
    assert np.array_equal(a["w"], b["w"])
    assert np.array_equal(a["sdf"], b["sdf"])


def test_batched_refusion_scattered_depths():
    """The batched collection off its common path (random depths up to 40 m:
    blocks beyond the tile set's key range, crowded tile sets) still gives the
    volume of the sequential calls bit for bit."""
    rows, cols = 48, 64
    rng = np.random.default_rng(11)
    depth = rng.integers(400, 40000, size=(6, rows, cols)).astype(np.uint16)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    intr = (52.5, 52.5, (cols - 1) / 2.0, (rows - 1) / 2.0)
    P = np.stack([np.eye(4)] * 6)
    P[:, 0, 3] = np.linspace(0, 0.2, 6)
    T_new = np.stack([delta(rng) @ P[k] for k in range(6)])
    out = []
    for batched in (False, True):
        g = GPUVoxelGrid(int(1e9), 0.016, 0.004, rows, cols, storage="f16", with_color=False, hash_buckets=1 << 19,
                         max_weight=255)
        g.setIntrinsic(*intr)
        for k in range(6):
            g.integrate_fast(dev[k], P[k].astype(np.float32))
        if batched:
            g.refuse_batch(dev, P, T_new)
        else:
            for k in range(6):
                g.integrate_fast(dev[k], P[k].astype(np.float32), deint=True)
                g.integrate_fast(dev[k], T_new[k].astype(np.float32))
        g.sync()
        out.append(g.export_blocks(with_color=False))
        g.close()
    a, b = out
    assert len(a["keys"]) > 10000
    assert np.array_equal(a["keys"], b["keys"]) and np.array_equal(a["coords"], b["coords"])
    assert np.array_equal(a["w"], b["w"]) and np.array_equal(a["sdf"], b["sdf"])


def test_batched_refusion_far_new_pose():
    """Keyframes re-fused at poses 25 m from the old ones: the new phase's
    blocks lie outside the tile set's key range (keys are offsets from the old
    pose's camera block), so they are visited one by one with that phase's bit;
    the volume still equals the sequential calls' bit for bit."""
    rows, cols = 48, 64
    rng = np.random.default_rng(12)
    depth = rng.integers(500, 4000, size=(6, rows, cols)).astype(np.uint16)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    intr = (52.5, 52.5, (cols - 1) / 2.0, (rows - 1) / 2.0)
    P = np.stack([np.eye(4)] * 6)
    P[:, 1, 3] = np.linspace(0, 0.2, 6)
    T_new = np.stack([delta(rng) @ P[k] for k in range(6)])
    T_new[::2, 0, 3] += 25.0  # keyframes 0, 2, 4 move 25 m along x
    out = []
    for batched in (False, True):
        g = GPUVoxelGrid(int(1e9), 0.016, 0.004, rows, cols, storage="f16", with_color=False, hash_buckets=1 << 18,
                         max_weight=255)
        g.setIntrinsic(*intr)
        for k in range(6):
            g.integrate_fast(dev[k], P[k].astype(np.float32))
        if batched:
            g.refuse_batch(dev, P, T_new)
        else:
            for k in range(6):
                g.integrate_fast(dev[k], P[k].astype(np.float32), deint=True)
                g.integrate_fast(dev[k], T_new[k].astype(np.float32))
        g.sync()
        out.append(g.export_blocks(with_color=False))
        g.close()
    a, b = out
    assert (a["coords"][:, 0] > 500).sum() > 100  # blocks near the moved poses (x > 16 m)
    assert np.array_equal(a["keys"], b["keys"]) and np.array_equal(a["coords"], b["coords"])
    assert np.array_equal(a["w"], b["w"]) and np.array_equal(a["sdf"], b["sdf"])
