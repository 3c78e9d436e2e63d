"""The integration thread's schedule (src/core/integrate.cpp:47-236) over
libss.so: frames queued for integration, re-integration when their pose
changes (largest change first, threshold treint) and deintegration; each step
fuses the new frames, re-fuses up to max_batch changed frames as one batched
re-fusion and deintegrates the removed ones, all stream-ordered."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import check, lib
from .voxel_grid import GPUVoxelGrid, _stream_ptr


def _d6(x) -> C.Array:
    a = np.asarray(x, np.float64).ravel()
    if a.size != 6:
        raise ValueError("expected 6 DoFs")
    return (C.c_double * 6)(*a)


def dofs_to_pose(dofs) -> np.ndarray:
    """getT (matrixutil.h:61-63): trans(t) Rz Ry Rx of (rx, ry, rz, tx, ty, tz)."""
    out = (C.c_double * 16)()
    check(lib.ss_dofs_to_pose(_d6(dofs), out), "dofs_to_pose")
    return np.array(out[:]).reshape(4, 4)


def pose_to_dofs(T) -> np.ndarray:
    """MattoDof (matrixutil.cpp:37-49)."""
    out = (C.c_double * 6)()
    check(lib.ss_pose_to_dofs((C.c_double * 16)(*np.asarray(T, np.float64).ravel()), out), "pose_to_dofs")
    return np.array(out[:])


def reintegration_order(world_dofs, integrated_dofs, treint: float) -> np.ndarray:
    """updateReintegrationBuffer's order of integrated frames (indices)."""
    w = np.ascontiguousarray(world_dofs, np.float64).reshape(-1, 6)
    i = np.ascontiguousarray(integrated_dofs, np.float64).reshape(-1, 6)
    n = len(w)
    order = np.zeros(max(n, 1), np.int32)
    cnt = C.c_int32()
    check(lib.ss_reintegration_order(n, C.c_void_p(w.ctypes.data), C.c_void_p(i.ctypes.data), float(treint),
                                     C.c_void_p(order.ctypes.data), C.byref(cnt)), "reintegration_order")
    return order[:cnt.value].copy()


class FusionScheduler:
    """pandia_integration's buffers for one grid (ids are the caller's; depth
    images are device tensors the caller keeps alive until deintegration)."""

    def __init__(self, grid: GPUVoxelGrid, treint: float = 0.04, max_batch: int = 64, exact: bool = False):
        self.grid = grid
        self._h = C.c_void_p()
        check(lib.ss_scheduler_create(grid.handle, float(treint), int(max_batch), 1 if exact else 0,
                                      C.byref(self._h)), "scheduler_create")
        self._depths = {}

    def close(self):
        if self._h:
            lib.ss_scheduler_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def push_integrate(self, frame_id: int, depth, dofs):
        check(lib.ss_scheduler_push_integrate(self._h, int(frame_id), C.c_void_p(depth.data_ptr()), _d6(dofs)),
              "scheduler_push_integrate")
        self._depths[int(frame_id)] = depth

    def set_dofs(self, frame_id: int, dofs):
        check(lib.ss_scheduler_set_dofs(self._h, int(frame_id), _d6(dofs)), "scheduler_set_dofs")

    def push_deintegrate(self, frame_id: int):
        check(lib.ss_scheduler_push_deintegrate(self._h, int(frame_id)), "scheduler_push_deintegrate")

    def update(self) -> int:
        q = C.c_int32()
        check(lib.ss_scheduler_update(self._h, C.byref(q)), "scheduler_update")
        return q.value

    def queue(self, which: str) -> list[int]:
        k = {"integrate": 0, "reintegrate": 1, "deintegrate": 2}[which]
        n = C.c_int32()
        check(lib.ss_scheduler_queue(self._h, k, 0, None, C.byref(n)), "scheduler_queue")
        ids = (C.c_int64 * max(n.value, 1))()
        check(lib.ss_scheduler_queue(self._h, k, n.value, ids, C.byref(n)), "scheduler_queue")
        return list(ids[:n.value])

    def step(self, stream=None) -> tuple[int, int, int]:
        done = (C.c_int32 * 3)()
        check(lib.ss_scheduler_step(self._h, _stream_ptr(stream), done), "scheduler_step")
        return tuple(done)

    def drain(self, stream=None) -> tuple[int, int, int]:
        done = (C.c_int32 * 3)()
        check(lib.ss_scheduler_drain(self._h, _stream_ptr(stream), done), "scheduler_drain")
        return tuple(done)

    def frame(self, frame_id: int):
        """(integrated, integrated DoFs)."""
        flag = C.c_int32()
        d = (C.c_double * 6)()
        check(lib.ss_scheduler_frame(self._h, int(frame_id), C.byref(flag), d), "scheduler_frame")
        return bool(flag.value), np.array(d[:])
