"""GPUVoxelGrid: the reference's voxel-hash TSDF interface over libss.so.

Mirrors ``GPUVoxelGrid`` (src/VoxelGrid/GPUVoxelGrid.h:40-120): same
constructor arguments ``(c, trunc, voxlength, resi, resj)``, same method
names and argument order (``integrate(rgb, depth, extr, withColor)``), same
outputs (``rayPcd`` / ``rayColorPcd`` owned by the grid, world coordinates).
Images are CUDA tensors in row-major ``[resi][resj]`` layout; poses are 4x4
camera->world matrices. Calls are asynchronous on the given stream (default:
torch's current stream); device-side errors surface at :meth:`sync`.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._native import (SS_STORAGE_F16, SS_STORAGE_F32, SSLaunchConfig, SSParams, check, f32x16, lib)

_STORAGE = {"f32": SS_STORAGE_F32, "f16": SS_STORAGE_F16}


def _stream_ptr(stream) -> C.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return C.c_void_p(stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))


def _dev_ptr(t: torch.Tensor, itemsize: int, shape: tuple, name: str) -> C.c_void_p:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if t.element_size() != itemsize or tuple(t.shape) != tuple(shape) or not t.is_contiguous():
        raise ValueError(f"{name}: expected contiguous {shape} with {itemsize}-byte elements, "
                         f"got {tuple(t.shape)} {t.dtype}")
    return C.c_void_p(t.data_ptr())


class GPUVoxelGrid:
    """Voxel-hash TSDF of 8^3 blocks (GPUVoxelGrid.h:40)."""

    def __init__(self, c: int, trunc: float, voxlength: float, resi_: int, resj_: int, *,
                 storage: str = "f32", with_color: bool = True, hash_buckets: int | None = None,
                 max_weight: float = 0.0, rmin: float = 0.2, d_max: float = 10.0, device=None):
        p = SSParams()
        check(lib.ss_params_default(C.byref(p), int(c), float(trunc), float(voxlength), int(resi_), int(resj_)),
              "ss_params_default")
        if hash_buckets is not None:
            p.hash_buckets = int(hash_buckets)
        p.storage = _STORAGE[storage]
        p.with_color = 1 if with_color else 0
        p.max_weight = float(max_weight)
        p.rmin = float(rmin)
        p.d_max = float(d_max)
        self.params = p
        self.d_trunc, self.vl, self.vbl = float(trunc), float(voxlength), 8.0 * float(voxlength)
        self.resi, self.resj = int(resi_), int(resj_)
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        self._h = C.c_void_p()
        with torch.cuda.device(self.device):
            check(lib.ss_grid_create(C.byref(p), C.byref(self._h)), "ss_grid_create")
            # raycast outputs owned by the grid, as rayPcd / rayColorPcd (GPUVoxelGrid.cpp:18-20)
            self.rayPcd = torch.zeros((self.resi, self.resj, 3), dtype=torch.float32, device=self.device)
            self.rayColorPcd = torch.zeros((self.resi, self.resj, 3), dtype=torch.float32, device=self.device)
        self.intrinsicSet = False

    # -- lifetime
    def close(self) -> None:
        if self._h:
            lib.ss_grid_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # -- reference methods
    def setIntrinsic(self, fx: float, fy: float, cx: float, cy: float) -> None:
        """setIntrinsic (GPUVoxelGrid.cpp:253-266); ci = resi - cy, cj = cx."""
        check(lib.ss_grid_set_intrinsic(self._h, float(fx), float(fy), float(cx), float(cy)), "setIntrinsic")
        self.intrinsicSet = True

    def _fuse(self, fn, name, rgb, depth, extr, withColor, stream):
        d = _dev_ptr(depth, 2, (self.resi, self.resj), "depth")
        r = _dev_ptr(rgb, 1, (self.resi, self.resj, 3), "rgb") if withColor else C.c_void_p()
        check(fn(self._h, d, r, f32x16(extr), 1 if withColor else 0, _stream_ptr(stream)), name)

    def integrate(self, rgb, depth, extr, withColor: bool = True, stream=None) -> None:
        """integrate (GPUVoxelGrid.cpp:41-83)."""
        self._fuse(lib.ss_integrate, "integrate", rgb, depth, extr, withColor, stream)

    def deIntegrate(self, rgb, depth, extr, withColor: bool = True, stream=None) -> None:
        """deIntegrate (GPUVoxelGrid.cpp:95-136)."""
        self._fuse(lib.ss_deintegrate, "deIntegrate", rgb, depth, extr, withColor, stream)

    def integrate_fast(self, depth, extr, deint: bool = False, rgb=None, stream=None) -> None:
        """The per-frame method's fusion (ss_integrate_fast): FMA arithmetic, nearest-pixel association."""
        d = _dev_ptr(depth, 2, (self.resi, self.resj), "depth")
        r = _dev_ptr(rgb, 1, (self.resi, self.resj, 3), "rgb") if rgb is not None else C.c_void_p()
        check(lib.ss_integrate_fast(self._h, d, r, f32x16(extr), 1 if rgb is not None else 0, 1 if deint else 0,
                                    _stream_ptr(stream)), "integrate_fast")

    def refuse_batch(self, depths, T_old, T_new, exact: bool = False, stream=None) -> None:
        """Re-fuse keyframes: for each k, deintegrate depths[k] at T_old[k] and integrate it at T_new[k]
        (in order), in one collection and one persistent apply launch. With no keyframes it only
        allocates the batch buffers (the first call on a grid does that otherwise)."""
        n = len(depths)
        for d in depths:
            _dev_ptr(d, 2, (self.resi, self.resj), "depth")
        ptrs = (C.c_void_p * n)(*[d.data_ptr() for d in depths])
        to = np.ascontiguousarray(np.asarray(T_old, np.float32).reshape(n, 16))
        tn = np.ascontiguousarray(np.asarray(T_new, np.float32).reshape(n, 16))
        check(lib.ss_refuse_batch(self._h, n, ptrs, C.c_void_p(to.ctypes.data), C.c_void_p(tn.ctypes.data),
                                  1 if exact else 0, _stream_ptr(stream)), "refuse_batch")

    def raycast(self, extr, stream=None, with_color: bool = True):
        """raycast (GPUVoxelGrid.cpp:139-147): fills rayPcd and rayColorPcd."""
        col = C.c_void_p(self.rayColorPcd.data_ptr()) if with_color else C.c_void_p()
        check(lib.ss_raycast(self._h, f32x16(extr), C.c_void_p(self.rayPcd.data_ptr()), col,
                             _stream_ptr(stream)), "raycast")
        return self.rayPcd, self.rayColorPcd

    def cleanMemory(self, stream=None) -> None:
        """cleanMemory (GPUVoxelGrid.cpp:185-196)."""
        check(lib.ss_clean_memory(self._h, _stream_ptr(stream)), "cleanMemory")

    # -- additions of the C-ABI
    LAUNCH_FIELDS = ("collect_rows", "raycast_rows", "fuse_ctas_per_sm", "refuse_ctas_per_sm", "track_ctas_per_sm")

    def launch_config(self) -> dict:
        c = SSLaunchConfig()
        check(lib.ss_grid_get_launch_config(self._h, C.byref(c)), "get_launch_config")
        return {f: getattr(c, f) for f in self.LAUNCH_FIELDS}

    def set_launch_config(self, **kw) -> None:
        cur = self.launch_config()
        cur.update(kw)
        c = SSLaunchConfig(*[int(cur[f]) for f in self.LAUNCH_FIELDS])
        check(lib.ss_grid_set_launch_config(self._h, C.byref(c)), "set_launch_config")

    def sync(self, stream=None) -> None:
        check(lib.ss_grid_sync(self._h, _stream_ptr(stream)), "sync")

    def reset(self, stream=None) -> None:
        check(lib.ss_grid_reset(self._h, _stream_ptr(stream)), "reset")

    def block_count(self, stream=None) -> int:
        n = C.c_int32()
        check(lib.ss_grid_block_count(self._h, _stream_ptr(stream), C.byref(n)), "block_count")
        return n.value

    def counters(self, stream=None) -> dict:
        a = (C.c_int64 * 6)()
        check(lib.ss_grid_counters(self._h, _stream_ptr(stream), a), "counters")
        return dict(live_blocks=a[0], last_touched=a[1], touched_total=a[2], calls=a[3], status=a[4],
                    epoch=a[5])

    def test_raycast_cap(self, cap: int) -> None:
        """Test hook: ss_raycast's per-ray iteration cap (0 restores the default)."""
        check(lib.ss_grid_test_raycast_cap(self._h, int(cap)), "test_raycast_cap")

    def raycast_counters(self, stream=None) -> dict:
        """Hash finds and voxel reads of every raycast call on this grid so far."""
        a = (C.c_int64 * 2)()
        check(lib.ss_grid_raycast_counters(self._h, _stream_ptr(stream), a), "raycast_counters")
        return dict(finds=a[0], voxels=a[1])

    def export_blocks(self, stream=None, with_color: bool = True) -> dict:
        """Canonical dump sorted by key (the host copy of marchingCubesHost, :204-206)."""
        n = C.c_int32()
        check(lib.ss_grid_export_blocks(self._h, _stream_ptr(stream), 0, None, None, None, None, None,
                                        C.byref(n)), "export_blocks")
        cap = n.value
        keys = np.zeros(cap, np.uint64)
        coords = np.zeros((cap, 3), np.int32)
        sdf = np.zeros((cap, 512), np.float32)
        w = np.zeros((cap, 512), np.float32)
        rgb = np.zeros((cap, 3, 512), np.float32) if with_color else None
        ptr = lambda a: C.c_void_p(a.ctypes.data) if a is not None and a.size else C.c_void_p()
        check(lib.ss_grid_export_blocks(self._h, _stream_ptr(stream), cap, ptr(keys), ptr(coords), ptr(sdf),
                                        ptr(w), ptr(rgb), C.byref(n)), "export_blocks")
        return dict(keys=keys, coords=coords, sdf=sdf, w=w, rgb=rgb)

    def export_buckets(self, stream=None) -> np.ndarray:
        """Bucket index of each block in export_blocks' (key) order."""
        n = C.c_int32()
        check(lib.ss_grid_export_buckets(self._h, _stream_ptr(stream), 0, None, C.byref(n)), "export_buckets")
        out = np.zeros(n.value, np.int32)
        check(lib.ss_grid_export_buckets(self._h, _stream_ptr(stream), n.value, C.c_void_p(out.ctypes.data),
                                          C.byref(n)), "export_buckets")
        return out

    def import_blocks(self, coords, sdf, w, rgb=None, stream=None) -> None:
        coords = np.ascontiguousarray(coords, np.int32)
        sdf = np.ascontiguousarray(sdf, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        rgbp = C.c_void_p(np.ascontiguousarray(rgb, np.float32).ctypes.data) if rgb is not None else C.c_void_p()
        check(lib.ss_grid_import_blocks(self._h, _stream_ptr(stream), len(coords), C.c_void_p(coords.ctypes.data),
                                        C.c_void_p(sdf.ctypes.data), C.c_void_p(w.ctypes.data), rgbp),
              "import_blocks")


def depth_to_pcd(depth: torch.Tensor, fx, fy, cx, cy, stream=None) -> torch.Tensor:
    """CreatePcdFromDepthView (imageutil.cpp:89-111)."""
    rows, cols = depth.shape
    out = torch.empty((rows, cols, 3), dtype=torch.float32, device=depth.device)
    check(lib.ss_depth_to_pcd(_dev_ptr(depth, 2, (rows, cols), "depth"), rows, cols, float(fx), float(fy),
                              float(cx), float(cy), C.c_void_p(out.data_ptr()), _stream_ptr(stream)),
          "depth_to_pcd")
    return out


def normals_from_pcd(pcd: torch.Tensor, stream=None) -> torch.Tensor:
    """CalculateNormalsFromPCDView (imageutil.cpp:117-157)."""
    rows, cols, _ = pcd.shape
    out = torch.empty_like(pcd)
    check(lib.ss_normals_from_pcd(_dev_ptr(pcd, 4, (rows, cols, 3), "pcd"), rows, cols,
                                  C.c_void_p(out.data_ptr()), _stream_ptr(stream)), "normals_from_pcd")
    return out
