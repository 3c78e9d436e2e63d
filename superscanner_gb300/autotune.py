"""Launch-shape autotuner for the reconstruction kernels.

Times candidate launch shapes on real frames and keeps the fastest, knob by
knob (coordinate descent): each knob is timed through the pipeline's own
stage profiler (CUDA events around collect, fuse, track and raycast of every
frame), the re-fusion knob through ss_refuse_batch. Results can be cached as
JSON keyed by GPU name, image size and storage form.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import torch

from .pipeline import Pipeline
from .voxel_grid import GPUVoxelGrid

CANDIDATES = {
    "raycast_rows": (2, 4, 8, 16),
    "collect_rows": (2, 4, 8),
    "fuse_ctas_per_sm": (4, 8, 16),
    "track_ctas_per_sm": (1, 2),
    "refuse_ctas_per_sm": (4, 8, 16),
}
STAGE = {"raycast_rows": "raycast", "collect_rows": "collect", "fuse_ctas_per_sm": "fuse",
         "track_ctas_per_sm": "track"}
DEFAULT = {"collect_rows": 8, "raycast_rows": 8, "fuse_ctas_per_sm": 8, "refuse_ctas_per_sm": 8,
           "track_ctas_per_sm": 2}


def _cache_key(rows: int, cols: int, storage: str) -> str:
    name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{name}|{rows}x{cols}|{storage}"


def _grid(grid_kw: dict, intr, cfg: dict) -> GPUVoxelGrid:
    g = GPUVoxelGrid(**grid_kw)
    g.setIntrinsic(*intr)
    g.set_launch_config(**cfg)
    return g


def _stage_ms(depth_dev, poses, frames: int, grid_kw: dict, intr, cfg: dict, pipe_kw: dict) -> dict:
    g = _grid(grid_kw, intr, cfg)
    pipe = Pipeline(g, use_graph=False, **pipe_kw)
    pipe.set_pose(poses[0])
    pipe.frame(depth_dev[0], track=False)
    pipe.frame(depth_dev[1])
    pipe.profile(True)
    for k in range(2, frames):
        pipe.frame(depth_dev[k])
    ms, n, _ = pipe.stage_ms()
    g.sync()
    pipe.close()
    g.close()
    return {k: v / max(n, 1) for k, v in ms.items()}


def _refuse_ms(depth_dev, poses, frames: int, grid_kw: dict, intr, cfg: dict) -> float:
    g = _grid(grid_kw, intr, cfg)
    for k in range(frames):
        g.integrate_fast(depth_dev[k], poses[k].astype(np.float32))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    kf = list(range(frames))
    e0.record()
    g.refuse_batch([depth_dev[k] for k in kf], poses[kf], poses[kf])
    e1.record()
    torch.cuda.synchronize()
    g.sync()
    g.close()
    return e0.elapsed_time(e1)


def autotune(depth_dev, poses, grid_kw: dict, intr, *, frames: int = 8, pipe_kw: dict | None = None,
             cache: str | Path | None = None, stage_timer=None, refuse_timer=None) -> dict:
    """Returns the launch configuration (GPUVoxelGrid.set_launch_config keywords).

    depth_dev: CUDA tensor [n, rows, cols] of frames along poses [n, 4, 4] (n >= frames).
    grid_kw: GPUVoxelGrid constructor keywords of the grid the result is for.
    Coordinate descent: the knobs are tuned one after the other in the order of
    CANDIDATES, each timed with the best values found so far for the earlier
    knobs and the defaults for the later ones; ties keep the first candidate.
    stage_timer(cfg) -> {stage: ms per frame} and refuse_timer(cfg) -> ms
    replace the GPU timings (the pipeline's stage profiler, one
    ss_refuse_batch call) when given.
    """
    pipe_kw = dict(pipe_kw or {})
    if stage_timer is None:
        stage_timer = lambda cfg: _stage_ms(depth_dev, poses, frames, grid_kw, intr, cfg, pipe_kw)  # noqa: E731
    if refuse_timer is None:
        refuse_timer = lambda cfg: _refuse_ms(depth_dev, poses, frames, grid_kw, intr, cfg)  # noqa: E731
    rows, cols = int(grid_kw["resi_"]), int(grid_kw["resj_"])
    key = _cache_key(rows, cols, grid_kw.get("storage", "f32"))
    if cache is not None and Path(cache).exists():
        stored = json.loads(Path(cache).read_text())
        if key in stored:
            return stored[key]["config"]
    best = dict(DEFAULT)
    timings = {}
    for knob, values in CANDIDATES.items():
        t = {}
        for v in values:
            cfg = dict(best, **{knob: v})
            if knob == "refuse_ctas_per_sm":
                t[v] = refuse_timer(cfg)
            else:
                t[v] = stage_timer(cfg)[STAGE[knob]]
        best[knob] = min(t, key=t.get)
        timings[knob] = {str(k): round(v, 5) for k, v in t.items()}
    if cache is not None:
        path = Path(cache)
        stored = json.loads(path.read_text()) if path.exists() else {}
        stored[key] = {"config": best, "ms": timings}
        path.write_text(json.dumps(stored, indent=1))
    best_with_timings = dict(best)
    best_with_timings["_ms"] = timings
    return best_with_timings
