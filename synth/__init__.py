"""Seeded synthetic RGB-D sequences (analytic rooms, spheres, boxes).

Stand-ins for the reference's recorded scenes, which are not available:
config-1 style rooms (2x2x2 m, 6 spheres + 4 boxes) and config-2 style rooms
(4x4x3 m, 40 primitives), smooth seeded trajectories, exact depth in uint16
millimetres with optional depth-dependent Gaussian noise and 5 % dropout.

Input data for tests and benchmarks, kept apart from the library package so
that loading it loads no part of the product. The C++ generator
(ss_synth.cpp) is compiled into _build/libss_synth.so on first import (or by
build()) with -ffp-contract=off, so x86 and Arm render the same frames.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
_SRC = _DIR / "ss_synth.cpp"
_LIB_PATH = _DIR / "_build" / "libss_synth.so"


def build(force: bool = False) -> Path:
    if force or not _LIB_PATH.exists() or _LIB_PATH.stat().st_mtime < _SRC.stat().st_mtime:
        _LIB_PATH.parent.mkdir(exist_ok=True)
        tmp = _LIB_PATH.with_suffix(f".so.tmp{os.getpid()}")
        subprocess.run(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
                        "-o", str(tmp), str(_SRC)], check=True)
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


build()
_lib = C.CDLL(str(_LIB_PATH))
_lib.synth_scene_new.restype = C.c_void_p
_lib.synth_scene_new.argtypes = [C.c_int, C.c_uint64]
_lib.synth_scene_free.argtypes = [C.c_void_p]
_lib.synth_num_primitives.restype = C.c_int
_lib.synth_num_primitives.argtypes = [C.c_void_p]
_lib.synth_primitives.argtypes = [C.c_void_p, C.c_void_p]
_lib.synth_trajectory.argtypes = [C.c_void_p, C.c_int, C.c_uint64, C.c_void_p]
_lib.synth_render.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_int, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p]

FX, FY, CX, CY = 525.0, 525.0, 319.5, 239.5
ROWS, COLS = 480, 640


class Scene:
    """kind 1: 2x2x2 m room, 6 spheres (r 0.1-0.4 m), 4 boxes; kind 2: 4x4x3 m, 40 primitives."""

    def __init__(self, kind: int = 1, seed: int = 1234):
        self.kind, self.seed = kind, seed
        self._h = _lib.synth_scene_new(kind, seed)

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.synth_scene_free(self._h)
            self._h = None

    def primitives(self) -> np.ndarray:
        n = _lib.synth_num_primitives(self._h)
        out = np.zeros((n, 11), np.float64)
        _lib.synth_primitives(self._h, out.ctypes.data)
        return out

    def trajectory(self, n: int, seed: int = 42) -> np.ndarray:
        poses = np.zeros((n, 4, 4), np.float64)
        _lib.synth_trajectory(self._h, n, seed, poses.ctypes.data)
        return poses

    def render(self, poses, rows: int = ROWS, cols: int = COLS, intr=(FX, FY, CX, CY), noise: bool = False,
               noise_seed: int = 7, frame0: int = 0, color: bool = True):
        poses = np.ascontiguousarray(np.asarray(poses, np.float64).reshape(-1, 4, 4))
        n = len(poses)
        depth = np.zeros((n, rows, cols), np.uint16)
        rgb = np.zeros((n, rows, cols, 3), np.uint8) if color else None
        _lib.synth_render(self._h, n, poses.ctypes.data, rows, cols, *map(float, intr), int(noise), noise_seed,
                          frame0, depth.ctypes.data, rgb.ctypes.data if color else None)
        return depth, rgb


def occlusion_masks(n: int, rows: int, cols: int, seed: int = 99, lo: float = 0.2, hi: float = 1.0):
    """Seeded rectangular occlusion masks keeping a 20-100 % share of each frame."""
    rng = np.random.default_rng(seed)
    masks = np.ones((n, rows, cols), bool)
    for k in range(n):
        keep = rng.uniform(lo, hi)
        if keep >= 0.999:
            continue
        area = 1.0 - keep
        h = int(np.clip(np.sqrt(area) * rows * rng.uniform(0.7, 1.3), 1, rows))
        w = int(np.clip(area * rows * cols / h, 1, cols))
        r0 = rng.integers(0, rows - h + 1)
        c0 = rng.integers(0, cols - w + 1)
        masks[k, r0:r0 + h, c0:c0 + w] = False
    return masks
