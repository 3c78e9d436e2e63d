"""Integration scheduling (src/core/integrate.cpp:47-236) on the host: the
DoF <-> pose conventions and the re-integration order of the library against
the oracle's restatement (no GPU)."""
import numpy as np

import oracle
from superscanner_gb300.scheduler import dofs_to_pose, pose_to_dofs, reintegration_order


def test_dofs_to_pose_matches_the_reference_product():
    rng = np.random.default_rng(0)
    for _ in range(50):
        x = np.concatenate([rng.uniform(-3, 3, 3), rng.uniform(-5, 5, 3)])
        assert np.abs(dofs_to_pose(x) - oracle.dofs_to_pose(x)).max() < 1e-14


def test_dofs_known_answer_and_round_trip():
    T = dofs_to_pose([0, 0, np.pi / 2, 1, 2, 3])
    assert np.allclose(T[:3, :3], [[0, -1, 0], [1, 0, 0], [0, 0, 1]], atol=1e-15)
    assert np.allclose(T[:3, 3], [1, 2, 3])
    rng = np.random.default_rng(1)
    for _ in range(50):
        x = np.concatenate([rng.uniform(-3, 3, 1), rng.uniform(-1.5, 1.5, 1), rng.uniform(-3, 3, 1),
                            rng.uniform(-5, 5, 3)])
        assert np.abs(pose_to_dofs(dofs_to_pose(x)) - x).max() < 1e-12
        assert np.abs(pose_to_dofs(dofs_to_pose(x)) - oracle.pose_to_dofs(oracle.dofs_to_pose(x))).max() < 1e-12


def test_reintegration_order_matches_the_oracle():
    rng = np.random.default_rng(2)
    for trial in range(20):
        n = int(rng.integers(0, 40))
        integ = rng.normal(size=(n, 6))
        world = integ + rng.normal(scale=0.03, size=(n, 6)) * (rng.random((n, 1)) < 0.7)
        if n > 3:  # an exact tie (identical frames) keeps integration order
            world[1], integ[1] = world[0], integ[0]
        treint = 0.04
        assert list(reintegration_order(world, integ, treint)) == oracle.reintegration_order(world, integ, treint)
    # a change of exactly treint is kept (the loop stops at diff < treint)
    w = np.zeros((2, 6))
    w[0, 3] = 0.02  # diff = 2 x 0.02 = 0.04
    assert list(reintegration_order(w, np.zeros((2, 6)), 0.04)) == [0]
