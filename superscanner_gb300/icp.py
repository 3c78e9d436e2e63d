"""kokkosICP over libss.so (src/postprocessing/kokkosICP.{h,cpp})."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._native import check, f64x16, lib
from .voxel_grid import _dev_ptr, _stream_ptr

PointToPoint, PointToPlane = 0, 1  # enum ICPTypes (kokkosICP.h:4-8)

# PrimeSense default intrinsic (the reference's g_intrinsic, coreutil.cpp:86-91)
PRIMESENSE = (525.0, 525.0, 319.5, 239.5)


def kokkos_icp(d1, d2, tx, ty, ICPType: int = PointToPoint, intrinsic=PRIMESENSE, stream=None):
    """kokkosICP(space, d1, d2, tx, ty, ICPType, &rmse) (kokkosICP.cpp:25-210).

    Aligns depth image ``d1`` (camera->world ``tx``) to ``d2`` (``ty``); returns
    ``(Txy, rmse)`` where ``Txy`` (4x4 float64) maps d1's camera frame into
    d2's, as the reference returns ``bestTxy_eigen`` and writes ``*rsme_extern``.
    """
    rows, cols = d1.shape
    out = (C.c_double * 16)()
    rmse = C.c_float()
    fx, fy, cx, cy = intrinsic
    check(lib.ss_kokkos_icp(_dev_ptr(d1, 2, (rows, cols), "d1"), _dev_ptr(d2, 2, (rows, cols), "d2"), rows, cols,
                            float(fx), float(fy), float(cx), float(cy), f64x16(tx), f64x16(ty), int(ICPType), out,
                            C.byref(rmse), _stream_ptr(stream)), "kokkosICP")
    return np.array(out[:], dtype=np.float64).reshape(4, 4), float(rmse.value)


def kokkos_icp_noalloc(d1, d2, tx, ty, ICPType: int = PointToPoint, intrinsic=PRIMESENSE, stream=None):
    """kokkos_icp through ss_kokkos_icp_noalloc: no device allocation, scratch in a
    fixed static device array (images up to 640 x 480; overlapping calls race)."""
    rows, cols = d1.shape
    out = (C.c_double * 16)()
    rmse = C.c_float()
    fx, fy, cx, cy = intrinsic
    check(lib.ss_kokkos_icp_noalloc(_dev_ptr(d1, 2, (rows, cols), "d1"), _dev_ptr(d2, 2, (rows, cols), "d2"), rows,
                                    cols, float(fx), float(fy), float(cx), float(cy), f64x16(tx), f64x16(ty),
                                    int(ICPType), out, C.byref(rmse), _stream_ptr(stream)), "kokkosICP (no alloc)")
    return np.array(out[:], dtype=np.float64).reshape(4, 4), float(rmse.value)
