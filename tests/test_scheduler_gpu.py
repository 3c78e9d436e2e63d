"""The integration schedule on the GPU: the scheduler's volume equals the
volume of the same integrations, re-integrations and deintegrations issued as
single calls (bit for bit: the batched re-fusion is exact), and its
re-integration queue follows the oracle's order."""
import numpy as np
import pytest
import torch

import oracle
import synth
from superscanner_gb300 import GPUVoxelGrid
from superscanner_gb300.scheduler import FusionScheduler, dofs_to_pose, pose_to_dofs

pytestmark = pytest.mark.gpu

INTR = (525.0, 525.0, 319.5, 239.5)
VL, TRUNC = 0.004, 0.016


def grid():
    g = GPUVoxelGrid(int(1e9), TRUNC, VL, 480, 640, storage="f16", with_color=False, hash_buckets=1 << 18,
                     max_weight=255)
    g.setIntrinsic(*INTR)
    return g


def f32_pose(dofs):
    return dofs_to_pose(dofs).astype(np.float32)


def test_scheduler_volume_equals_single_calls():
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(30, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, noise_seed=7, color=False)
    dev = [torch.from_numpy(np.ascontiguousarray(d.view(np.int16))).cuda() for d in depth]
    dofs = [pose_to_dofs(T) for T in P]
    g = grid()
    S = FusionScheduler(g, treint=0.04, max_batch=8)
    for k in range(30):
        S.push_integrate(k, dev[k], dofs[k])
    assert S.step() == (30, 0, 0)
    # a pose optimisation moves 16 frames, some by less than the threshold
    rng = np.random.default_rng(4)
    world = [d.copy() for d in dofs]
    for k in rng.choice(30, 16, replace=False):
        step = rng.normal(size=6) * np.array([0.01, 0.01, 0.01, 0.008, 0.008, 0.008]) * rng.uniform(0.2, 3.0)
        world[k] = dofs[k] + step
        S.set_dofs(int(k), world[k])
    queued = S.update()
    order = S.queue("reintegrate")
    assert order == oracle.reintegration_order(world, dofs, 0.04)
    assert 8 < queued < 16
    # deintegrating a queued frame takes it off the re-integration queue
    gone = order[-1]
    S.push_deintegrate(gone)
    assert gone not in S.queue("reintegrate")
    order = order[:-1]
    # a frame removed before its integration is just dropped
    S.push_integrate(99, dev[0], dofs[0])
    S.push_deintegrate(99)
    assert S.queue("integrate") == []
    assert S.step() == (0, 8, 1)
    assert S.step() == (0, len(order) - 8, 0)
    for k in order:
        flag, d = S.frame(k)
        assert flag and np.array_equal(d, world[k])
    S.push_deintegrate(29)
    assert S.drain() == (0, 0, 1)

    # the same work as single calls on a second grid
    g2 = grid()
    for k in range(30):
        g2.integrate_fast(dev[k], f32_pose(dofs[k]))
    def refuse(ks):
        for k in ks:
            g2.integrate_fast(dev[k], f32_pose(dofs[k]), deint=True)
            g2.integrate_fast(dev[k], f32_pose(world[k]))
    refuse(order[:8])  # step 1: a batch of 8 re-fusions, then the deintegration
    g2.integrate_fast(dev[gone], f32_pose(dofs[gone]), deint=True)
    refuse(order[8:])  # step 2
    g2.integrate_fast(dev[29], f32_pose(world[29]), deint=True)  # the drain
    g.sync()
    g2.sync()
    a, b = g.export_blocks(with_color=False), g2.export_blocks(with_color=False)
    assert np.array_equal(a["keys"], b["keys"])
    assert np.array_equal(a["w"], b["w"]) and np.array_equal(a["sdf"], b["sdf"])
    S.close()
