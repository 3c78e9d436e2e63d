"""The reference's own hot-path code on the CPU — test infrastructure only.

Loads ``oracle/_ref/libss_ref.so``: the reference's unmodified
GPUVoxelGrid.cpp, kokkosICP.cpp, imageutil.cpp, kokkosUtil.cpp and
kokkosFunctions.cpp compiled by ``make -C oracle ref`` against the stand-ins
of ``oracle/ref_stub/`` (Kokkos, Eigen, Open3D, OpenCV), with the C entry
points of ``oracle/ref_driver.cpp``. The library is built from the reference
checkout, so it exists only where that checkout does; ``available()`` says
whether it could be loaded. ``tests/golden/make_ref_golden.py`` freezes its
outputs into the committed fixtures that pin the oracle and the CUDA path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
REF_ROOT = Path(os.environ.get("SS_REFERENCE", "/root/reference"))
_LIBS = {False: _DIR / "_ref" / "libss_ref.so", True: _DIR / "_ref" / "libss_ref_fma.so"}
_loaded: dict = {}


def build(force: bool = False) -> bool:
    """Compiles oracle/_ref when the reference checkout is present; True if the library exists."""
    if (REF_ROOT / "src" / "VoxelGrid" / "GPUVoxelGrid.cpp").exists():
        subprocess.run(["make", "-s", *(["-B"] if force else []), "-C", str(_DIR), "ref", f"REF={REF_ROOT}"],
                       check=True)
    return _LIBS[False].exists()


def available(fma: bool = False) -> bool:
    return _LIBS[fma].exists()


def _lib(fma: bool = False):
    if fma in _loaded:
        return _loaded[fma]
    lib = C.CDLL(str(_LIBS[fma]))
    p, i, f = C.c_void_p, C.c_int, C.c_float
    for name, res, args in [
        ("ssref_grid_new", p, [C.c_uint, f, f, i, i]),
        ("ssref_grid_free", None, [p]),
        ("ssref_set_intrinsic", None, [p, f, f, f, f]),
        ("ssref_fuse", None, [p, p, p, p, i, i]),
        ("ssref_raycast", None, [p, p, p, p]),
        ("ssref_clean", None, [p]),
        ("ssref_count", i, [p]),
        ("ssref_dump", i, [p, i, p, p, p, p, p, p]),
        ("ssref_mc_units", i, [p, i, p, p, p]),
        ("ssref_depth_to_pcd", None, [p, i, i, f, f, f, f, p]),
        ("ssref_normals", None, [p, i, i, p]),
        ("ssref_kokkos_icp", None, [p, p, i, i, f, f, f, f, p, p, i, p, p]),
    ]:
        fn = getattr(lib, name)
        fn.restype, fn.argtypes = res, args
    _loaded[fma] = lib
    return lib


def _ptr(a):
    return a.ctypes if a is not None else C.c_void_p()


class RefGrid:
    """GPUVoxelGrid itself (the reference's class, run serially on the host)."""

    def __init__(self, vl, trunc, resi, resj, intr=(525.0, 525.0, 319.5, 239.5), capacity_voxels=1 << 27,
                 fma=False):
        self.resi, self.resj = resi, resj
        self._l = _lib(fma)
        self._h = self._l.ssref_grid_new(int(capacity_voxels), float(trunc), float(vl), resi, resj)
        self._l.ssref_set_intrinsic(self._h, *map(float, intr))

    def __del__(self):
        if getattr(self, "_h", None):
            self._l.ssref_grid_free(self._h)
            self._h = None

    def fuse(self, depth, rgb, extr, with_color=True, deint=False):
        depth = np.ascontiguousarray(depth, np.uint16)
        rgb = np.ascontiguousarray(rgb, np.uint8) if rgb is not None else None
        E = np.ascontiguousarray(extr, np.float32).reshape(16)
        self._l.ssref_fuse(self._h, _ptr(depth), _ptr(rgb), _ptr(E), int(bool(with_color)), int(bool(deint)))

    def integrate(self, depth, rgb, extr, with_color=True):
        self.fuse(depth, rgb, extr, with_color, False)

    def deintegrate(self, depth, rgb, extr, with_color=True):
        self.fuse(depth, rgb, extr, with_color, True)

    def clean(self):
        self._l.ssref_clean(self._h)

    def count(self) -> int:
        return self._l.ssref_count(self._h)

    def export(self) -> dict:
        """Live entries sorted by key: keys, coords (vbInd), pzero, sdf, w, rgb."""
        n = self.count()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        pzero = np.zeros((n, 3), np.float32)
        sdf = np.zeros((n, 512), np.float32)
        w = np.zeros((n, 512), np.int16)
        rgb = np.zeros((n, 3, 512), np.float32)
        m = self._l.ssref_dump(self._h, n, _ptr(keys), _ptr(coords), _ptr(pzero), _ptr(sdf), _ptr(w), _ptr(rgb))
        assert m == n
        o = np.argsort(keys, kind="stable")
        return dict(keys=keys[o], coords=coords[o], pzero=pzero[o], sdf=sdf[o], w=w[o], rgb=rgb[o])

    def raycast(self, extr):
        pcd = np.zeros((self.resi, self.resj, 3), np.float32)
        col = np.zeros((self.resi, self.resj, 3), np.float32)
        E = np.ascontiguousarray(extr, np.float32).reshape(16)
        self._l.ssref_raycast(self._h, _ptr(E), _ptr(pcd), _ptr(col))
        return pcd, col

    def marching_cubes_units(self) -> dict:
        """The Open3D volume units marchingCubesHost fills, sorted by unit index."""
        n = self.count()
        index = np.zeros((n, 3), np.int32)
        tsdf = np.zeros((n, 512), np.float32)
        weight = np.zeros((n, 512), np.float32)
        m = self._l.ssref_mc_units(self._h, n, _ptr(index), _ptr(tsdf), _ptr(weight))
        o = np.lexsort((index[:m, 2], index[:m, 1], index[:m, 0]))
        return dict(index=index[:m][o], tsdf=tsdf[:m][o], weight=weight[:m][o])


def depth_to_pcd(depth, intr=(525.0, 525.0, 319.5, 239.5)):
    depth = np.ascontiguousarray(depth, np.uint16)
    rows, cols = depth.shape
    out = np.zeros((rows, cols, 3), np.float32)
    _lib().ssref_depth_to_pcd(_ptr(depth), rows, cols, *map(float, intr), _ptr(out))
    return out


def normals(pcd):
    pcd = np.ascontiguousarray(pcd, np.float32)
    rows, cols, _ = pcd.shape
    out = np.zeros_like(pcd)
    _lib().ssref_normals(_ptr(pcd), rows, cols, _ptr(out))
    return out


def kokkos_icp(d1, d2, tx, ty, icp_type=0, intr=(525.0, 525.0, 319.5, 239.5), fma=False):
    d1 = np.ascontiguousarray(d1, np.uint16)
    d2 = np.ascontiguousarray(d2, np.uint16)
    rows, cols = d1.shape
    out = np.zeros(16)
    rmse = np.zeros(1, np.float32)
    _lib(fma).ssref_kokkos_icp(_ptr(d1), _ptr(d2), rows, cols, *map(float, intr),
                               _ptr(np.ascontiguousarray(tx, np.float64)), _ptr(np.ascontiguousarray(ty, np.float64)),
                               int(icp_type), _ptr(out), _ptr(rmse))
    return out.reshape(4, 4), float(rmse[0])
