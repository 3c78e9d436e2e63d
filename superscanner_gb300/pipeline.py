"""Per-frame reconstruction pipeline over libss.so: track the frame against
the last model view (3-level point-to-plane Gauss-Newton), integrate it at
the tracked pose, raycast the new model view (trilinear, <= 128 steps).

Forms: ``plain`` = FP32 TSDF, every kernel launched one by one (one launch
per tracker iteration); ``chosen`` = FP16 TSDF + uint16 weights, all tracker
iterations in one persistent cooperative launch, each tracked frame replayed
as one CUDA graph. Both keep all state on the device (no host sync per frame).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._native import SSPipelineParams, check, f32x16, f64x16, lib
from .voxel_grid import GPUVoxelGrid, _stream_ptr


def raycast_maps(grid: GPUVoxelGrid, extr, max_steps: int = 128, t_min: float = 0.2, t_max: float = 10.0,
                 hint_depth=None, hint_margin: float = 0.0, stream=None):
    """Trilinear raycast: (vertex_depth [H,W,4], normal [H,W,4]) CUDA tensors."""
    vmap = torch.empty((grid.resi, grid.resj, 4), dtype=torch.float32, device=grid.device)
    nmap = torch.empty_like(vmap)
    hint = C.c_void_p(hint_depth.data_ptr()) if hint_depth is not None else C.c_void_p()
    check(lib.ss_raycast_maps(grid.handle, f32x16(extr), int(max_steps), float(t_min), float(t_max), hint,
                              float(hint_margin), C.c_void_p(vmap.data_ptr()), C.c_void_p(nmap.data_ptr()),
                              _stream_ptr(stream)), "raycast_maps")
    return vmap, nmap


FORMS = {
    "plain": dict(storage="f32", use_graph=False, persistent_track=False),
    "chosen": dict(storage="f16", use_graph=True, persistent_track=True),
}


class Pipeline:
    def __init__(self, grid: GPUVoxelGrid, *, use_graph: bool = True, levels: int = 3, iters=(10, 5, 4),
                 dist=(0.06, 0.10, 0.15), raycast_steps: int = 128, t_min: float = 0.2, t_max: float = 10.0,
                 exact_fusion: bool = False, hint_margin: float = 0.04, persistent_track: bool | None = None):
        p = SSPipelineParams()
        check(lib.ss_pipeline_params_default(C.byref(p)), "pipeline_params_default")
        p.levels = levels
        for k in range(4):
            p.iters[k] = int(iters[k]) if k < len(iters) else 0
            p.dist_thresh[k] = float(dist[k]) if k < len(dist) else 0.2
        p.raycast_steps = int(raycast_steps)
        p.t_min, p.t_max = float(t_min), float(t_max)
        p.use_graph = 1 if use_graph else 0
        p.exact_fusion = 1 if exact_fusion else 0
        p.hint_margin = float(hint_margin)
        p.persistent_track = int(use_graph if persistent_track is None else persistent_track)
        self.grid = grid
        self._h = C.c_void_p()
        check(lib.ss_pipeline_create(grid.handle, C.byref(p), C.byref(self._h)), "pipeline_create")
        ptr = C.c_void_p()
        check(lib.ss_pipeline_input(self._h, C.byref(ptr)), "pipeline_input")
        self.input_ptr = ptr.value

    def close(self):
        if self._h:
            lib.ss_pipeline_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_pose(self, T, stream=None):
        check(lib.ss_pipeline_set_pose(self._h, f64x16(T), _stream_ptr(stream)), "pipeline_set_pose")

    def set_start(self, T, stream=None):
        """One-shot ICP start pose for the next tracked frame (the model maps stay at the current pose)."""
        check(lib.ss_pipeline_set_start(self._h, f64x16(T), _stream_ptr(stream)), "pipeline_set_start")

    def pose(self, stream=None) -> np.ndarray:
        out = (C.c_double * 16)()
        check(lib.ss_pipeline_get_pose(self._h, out, _stream_ptr(stream)), "pipeline_get_pose")
        return np.array(out[:], np.float64).reshape(4, 4)

    def read_pose_async(self, dst_ptr: int, stream=None):
        """Enqueue the pose (16 doubles) into dst_ptr (pinned host or device) without a host sync."""
        check(lib.ss_pipeline_read_pose(self._h, C.c_void_p(dst_ptr), _stream_ptr(stream)), "pipeline_read_pose")

    def frame(self, depth, track: bool = True, stream=None):
        """depth: CUDA tensor [H, W] of 2-byte elements, pinned/host numpy uint16 array, or an int pointer."""
        if isinstance(depth, torch.Tensor):
            ptr = depth.data_ptr()
        elif isinstance(depth, np.ndarray):
            ptr = depth.ctypes.data
        else:
            ptr = int(depth)
        check(lib.ss_pipeline_frame(self._h, C.c_void_p(ptr), 1 if track else 0, _stream_ptr(stream)),
              "pipeline_frame")

    def maps(self):
        v, n = C.c_void_p(), C.c_void_p()
        check(lib.ss_pipeline_maps(self._h, C.byref(v), C.byref(n)), "pipeline_maps")
        return v.value, n.value

    def maps_tensors(self, stream=None):
        """Copies of the model maps as (vertex_depth, normal) CUDA tensors [H, W, 4]."""
        H, W = self.grid.resi, self.grid.resj
        out_v = torch.empty((H, W, 4), dtype=torch.float32, device=self.grid.device)
        out_n = torch.empty_like(out_v)
        check(lib.ss_pipeline_copy_maps(self._h, C.c_void_p(out_v.data_ptr()), C.c_void_p(out_n.data_ptr()),
                                        _stream_ptr(stream)), "pipeline_copy_maps")
        return out_v, out_n

    def profile(self, enable: bool = True):
        check(lib.ss_pipeline_profile(self._h, 1 if enable else 0), "pipeline_profile")

    STAGES = ("track", "collect", "fuse", "finalize", "raycast")

    def stage_ms(self, stream=None) -> tuple[dict, int, dict]:
        """(summed ms per stage, profiled frames, raycast counters)."""
        ms = (C.c_double * 5)()
        n = C.c_int64()
        cnt = (C.c_int64 * 4)()
        check(lib.ss_pipeline_stage_ms(self._h, ms, C.byref(n), cnt, _stream_ptr(stream)), "pipeline_stage_ms")
        rc = dict(zip(("lookups", "voxels", "steps", "hits"), list(cnt)))
        return dict(zip(self.STAGES, list(ms))), n.value, rc

    def stats(self, stream=None):
        inl = (C.c_int32 * 4)()
        rm = (C.c_float * 4)()
        check(lib.ss_pipeline_stats(self._h, inl, rm, _stream_ptr(stream)), "pipeline_stats")
        return list(inl), list(rm)

    def test_wait_timeout(self, polls: int = 1000):
        """Test hook: the next tracked frame's tracker wait runs out after `polls` polls
        (SS_ERR_TIMEOUT at the next sync; the frame keeps its start pose)."""
        check(lib.ss_pipeline_test_wait_timeout(self._h, int(polls)), "pipeline_test_wait_timeout")
