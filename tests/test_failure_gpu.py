"""Failure paths of the bounded device loops, made to run out through test
hooks (no fault, trap or endless loop): the kernel gives up within its limit,
the host reads SS_ERR_TIMEOUT at the next sync, and the GPU context and the
grid stay usable.

  * ss_raycast's per-ray iteration guard (raycastingTag's march,
    GPUVoxelGrid.cpp:561-715, has no bound; the library caps it at 2^20):
    a cap of a few iterations ends the long rays without a hit.
  * The persistent tracker's wait for the other CTAs' fixed-point sums (at
    most 2^22 polls): the test hook makes it wait for one contribution more
    than the CTAs make, for 1000 polls.
"""
import numpy as np
import pytest
import torch

import oracle
import synth
from superscanner_gb300 import GPUVoxelGrid
from superscanner_gb300._native import SS_ERR_TIMEOUT, SSError
from superscanner_gb300.pipeline import Pipeline

pytestmark = pytest.mark.gpu

INTR = (525.0, 525.0, 319.5, 239.5)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a.view(np.int16) if a.dtype == np.uint16 else a)).cuda()


def test_reference_raycast_iteration_cap_times_out_and_recovers():
    sc = synth.Scene(1, 1234)
    P = sc.trajectory(6, 42)[::2]
    depth, rgb = sc.render(P, 480, 640, INTR)
    g = GPUVoxelGrid(int(1e8), 0.02, 0.005, 480, 640, hash_buckets=1 << 16)
    g.setIntrinsic(*INTR)
    o = oracle.OracleGrid(0.005, 0.02, 480, 640, intr=INTR)
    for k in range(len(P)):
        g.integrate(dev(rgb[k]), dev(depth[k]), P[k].astype(np.float32))
        o.integrate(depth[k], rgb[k], P[k].astype(np.float32))
    g.sync()
    E = P[-1].astype(np.float32)
    op, _ = o.raycast(E)

    g.test_raycast_cap(12)  # a ray needs tens of block steps to reach the room's surfaces
    pcd, _ = g.raycast(E)
    with pytest.raises(SSError) as ei:
        g.sync()
    assert ei.value.code == SS_ERR_TIMEOUT
    capped = pcd.cpu().numpy()
    hit = capped[..., 2] != 0
    assert hit.mean() < 0.5 * (op[..., 2] != 0).mean()  # most rays ran out
    assert np.array_equal(capped[hit], op[hit])  # the rays that finished are the reference's

    g.test_raycast_cap(0)  # default cap: the same call is complete and exact again
    pcd, _ = g.raycast(E)
    g.sync()
    assert np.all(pcd.cpu().numpy() == op, axis=-1).mean() >= 0.999
    g.close()


def test_tracker_wait_times_out_and_the_next_frame_tracks():
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(8, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, color=False)
    g = GPUVoxelGrid(int(1e9), 0.016, 0.004, 480, 640, storage="f16", with_color=False, hash_buckets=1 << 18,
                     max_weight=255)
    g.setIntrinsic(*INTR)
    pipe = Pipeline(g, use_graph=True, persistent_track=True, hint_margin=0.04)
    d = dev(depth)
    pipe.set_pose(P[0])
    pipe.frame(d[0], track=False)
    for k in (1, 2, 3):
        pipe.frame(d[k])
    g.sync()
    before = pipe.pose()

    pipe.test_wait_timeout(1000)
    pipe.frame(d[4])
    with pytest.raises(SSError) as ei:
        g.sync()
    assert ei.value.code == SS_ERR_TIMEOUT
    assert np.array_equal(pipe.pose(), before)  # no CTA updated the pose: the frame kept its start

    for k in (5, 6, 7):  # the hook was one-shot: tracking resumes (through the graph again)
        pipe.frame(d[k])
    g.sync()
    dlt = np.linalg.inv(P[7]) @ pipe.pose()
    assert np.linalg.norm(dlt[:3, 3]) < 5e-3
    assert np.degrees(np.arccos(np.clip((np.trace(dlt[:3, :3]) - 1) / 2, -1, 1))) < 0.5
    torch.cuda.synchronize()
    assert torch.ones(4, device="cuda").sum().item() == 4.0  # the context is intact
    pipe.close()
    g.close()


def test_launch_config_change_recaptures_the_frame_graph():
    """A launch-shape change after the per-frame graphs were captured reaches
    graph frames too: the frame's result equals a direct-launch pipeline's
    with the same shapes."""
    sc = synth.Scene(2, 1234)
    P = sc.trajectory(8, 42)
    depth, _ = sc.render(P, 480, 640, INTR, noise=True, color=False)
    d = dev(depth)
    poses = []
    for graph in (True, False):
        g = GPUVoxelGrid(int(1e9), 0.016, 0.004, 480, 640, storage="f16", with_color=False, hash_buckets=1 << 18,
                         max_weight=255)
        g.setIntrinsic(*INTR)
        pipe = Pipeline(g, use_graph=graph, persistent_track=True, hint_margin=0.04)
        pipe.set_pose(P[0])
        pipe.frame(d[0], track=False)
        for k in range(1, 4):
            pipe.frame(d[k])
        g.set_launch_config(track_ctas_per_sm=1, collect_rows=4, raycast_rows=2)
        for k in range(4, 8):
            pipe.frame(d[k])
        g.sync()
        poses.append(pipe.pose())
        pipe.close()
        g.close()
    assert np.array_equal(poses[0], poses[1])
