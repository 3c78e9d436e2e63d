"""CPU oracle of the reconstruction hot path — test infrastructure only.

Loads ``oracle/_build/libss_oracle.so`` (built from ss_oracle.cpp by the
Makefile beside it). Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline legs use this module; the product package never imports it.
Parity status: pinned by the reference's own code (oracle/_ref, see
ss_oracle.cpp's header and tests/test_ref_pinned.py).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
_LIB_PATH = _DIR / "_build" / "libss_oracle.so"


def build(force: bool = False) -> Path:
    srcs = list(_DIR.glob("*.cpp")) + list(_DIR.glob("*.h")) + [_DIR / "Makefile"]
    if force or not _LIB_PATH.exists() or _LIB_PATH.stat().st_mtime < max(p.stat().st_mtime for p in srcs):
        subprocess.run(["make", "-s", "-B" if force else "-s", "-C", str(_DIR)], check=True)
    return _LIB_PATH


build()
_lib = C.CDLL(str(_LIB_PATH))
_p, _i, _f = C.c_void_p, C.c_int, C.c_float
for name, res, args in [
    ("orc_grid_new", _p, [_f, _f, _i, _i, _f]),
    ("orc_grid_free", None, [_p]),
    ("orc_grid_set_intrinsic", None, [_p, _f, _f, _f, _f]),
    ("orc_grid_fuse", _i, [_p, _p, _p, _p, _i, _i]),
    ("orc_grid_count", _i, [_p]),
    ("orc_grid_export", _i, [_p, _i, _p, _p, _p, _p, _p]),
    ("orc_grid_import", None, [_p, _i, _p, _p, _p, _p]),
    ("orc_grid_clean", _i, [_p]),
    ("orc_grid_raycast", None, [_p, _p, _p, _p]),
    ("orc_depth_to_pcd", None, [_p, _i, _i, _f, _f, _f, _f, _p]),
    ("orc_normals", None, [_p, _i, _i, _p]),
    ("orc_kokkos_icp", _i, [_p, _p, _i, _i, _f, _f, _f, _f, _p, _p, _i, _p, _p, _p]),
    ("orc_svd3", None, [_p, _p, _p, _p]),
    ("orc_inverse4f", None, [_p, _p]),
    ("orc_mat4_vec4", None, [_p, _p, _p]),
    ("orc_threads", _i, []),
    ("orm_grid_new", _p, [_f, _f, _i, _i, _f, _f, _f, _f, C.c_double]),
    ("orm_grid_free", None, [_p]),
    ("orm_grid_count", _i, [_p]),
    ("orm_grid_set_round_pixel", None, [_p, _i]),
    ("orm_grid_fuse", _i, [_p, _p, _p, _i]),
    ("orm_grid_export", _i, [_p, _i, _p, _p, _p, _p]),
    ("orm_raycast", None, [_p, _p, _i, C.c_double, C.c_double, _p, C.c_double, _p, _p, _p]),
    ("orm_track_debug", None, [_p, C.c_double]),
    ("orm_grid_import", None, [_p, _i, _p, _p, _p]),
    ("orm_grid_add_voxel", _i, [_p, _i, _i, _i, _i, C.c_double]),
    ("orm_raycast_loss_grad", C.c_double, [_p, _p, _p, C.c_double, C.c_double, _i, C.c_double, C.c_double, _p, _p]),
    ("orm_extract_mesh", C.c_longlong, [_p, C.c_longlong, _p]),
    ("orm_extract_mesh_cubes", C.c_longlong, [_p, C.c_longlong, _p]),
    ("orm_raycast_loss", C.c_double, [_p, _p, _p, C.c_double, C.c_double, _i, C.c_double, C.c_double, _p]),
    ("orm_raycast_loss_pixels", C.c_double, [_p, _p, _p, C.c_double, C.c_double, _i, C.c_double, C.c_double, _p,
                                             _p, _p]),
    ("orm_track", _i, [_p, _i, _i, _f, _f, _f, _f, _p, _p, _p, _p, _i, _p, _p, C.c_double, C.c_double]),
]:
    fn = getattr(_lib, name)
    fn.restype = res
    fn.argtypes = args


def _ptr(a):
    # numpy's ctypes view holds a reference to the array, so a temporary
    # (a converted copy) stays alive for the duration of the foreign call
    return a.ctypes if a is not None else C.c_void_p()


def _f32(a, shape=None):
    a = np.ascontiguousarray(a, np.float32)
    if shape is not None:
        a = a.reshape(shape)
    return a


class OracleGrid:
    """Reference-semantics voxel grid (GPUVoxelGrid restated on the CPU)."""

    def __init__(self, vl, trunc, resi, resj, intr=(525.0, 525.0, 319.5, 239.5), max_weight=0.0):
        self.resi, self.resj = resi, resj
        self._h = _lib.orc_grid_new(vl, trunc, resi, resj, max_weight)
        _lib.orc_grid_set_intrinsic(self._h, *map(float, intr))

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.orc_grid_free(self._h)
            self._h = None

    def fuse(self, depth, rgb, extr, with_color=True, deint=False) -> int:
        depth = np.ascontiguousarray(depth, np.uint16)
        rgb = np.ascontiguousarray(rgb, np.uint8) if (with_color and rgb is not None) else None
        E = _f32(extr, (16,))
        return _lib.orc_grid_fuse(self._h, _ptr(depth), _ptr(rgb), _ptr(E), int(with_color and rgb is not None),
                                  int(deint))

    def integrate(self, depth, rgb, extr, with_color=True):
        return self.fuse(depth, rgb, extr, with_color, False)

    def deintegrate(self, depth, rgb, extr, with_color=True):
        return self.fuse(depth, rgb, extr, with_color, True)

    def count(self) -> int:
        return _lib.orc_grid_count(self._h)

    def export(self) -> dict:
        n = self.count()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        sdf = np.zeros((n, 512), np.float32)
        w = np.zeros((n, 512), np.float32)
        rgb = np.zeros((n, 3, 512), np.float32)
        _lib.orc_grid_export(self._h, n, _ptr(keys), _ptr(coords), _ptr(sdf), _ptr(w), _ptr(rgb))
        return dict(keys=keys, coords=coords, sdf=sdf, w=w, rgb=rgb)

    def import_blocks(self, coords, sdf, w, rgb=None):
        coords = np.ascontiguousarray(coords, np.int32)
        _lib.orc_grid_import(self._h, len(coords), _ptr(coords), _ptr(_f32(sdf)), _ptr(_f32(w)),
                             _ptr(_f32(rgb)) if rgb is not None else C.c_void_p())

    def clean(self) -> int:
        return _lib.orc_grid_clean(self._h)

    def raycast(self, extr):
        pcd = np.zeros((self.resi, self.resj, 3), np.float32)
        col = np.zeros((self.resi, self.resj, 3), np.float32)
        _lib.orc_grid_raycast(self._h, _ptr(_f32(extr, (16,))), _ptr(pcd), _ptr(col))
        return pcd, col


def depth_to_pcd(depth, intr=(525.0, 525.0, 319.5, 239.5)):
    depth = np.ascontiguousarray(depth, np.uint16)
    rows, cols = depth.shape
    out = np.zeros((rows, cols, 3), np.float32)
    _lib.orc_depth_to_pcd(_ptr(depth), rows, cols, *map(float, intr), _ptr(out))
    return out


def normals(pcd):
    pcd = _f32(pcd)
    rows, cols, _ = pcd.shape
    out = np.zeros_like(pcd)
    _lib.orc_normals(_ptr(pcd), rows, cols, _ptr(out))
    return out


def kokkos_icp(d1, d2, tx, ty, icp_type=0, intr=(525.0, 525.0, 319.5, 239.5)):
    d1 = np.ascontiguousarray(d1, np.uint16)
    d2 = np.ascontiguousarray(d2, np.uint16)
    rows, cols = d1.shape
    tx = np.ascontiguousarray(tx, np.float64)
    ty = np.ascontiguousarray(ty, np.float64)
    out = np.zeros(16, np.float64)
    rmse = np.zeros(1, np.float32)
    stats = np.zeros((10, 4), np.float64)
    _lib.orc_kokkos_icp(_ptr(d1), _ptr(d2), rows, cols, *map(float, intr), _ptr(tx), _ptr(ty), int(icp_type),
                        _ptr(out), _ptr(rmse), _ptr(stats))
    return out.reshape(4, 4), float(rmse[0]), stats


def svd3(H):
    H = np.ascontiguousarray(H, np.float64)
    U = np.zeros(9)
    S = np.zeros(3)
    V = np.zeros(9)
    _lib.orc_svd3(_ptr(H), _ptr(U), _ptr(S), _ptr(V))
    return U.reshape(3, 3), S, V.reshape(3, 3)


def inverse4f(E):
    out = np.zeros(16, np.float32)
    _lib.orc_inverse4f(_ptr(_f32(E, (16,))), _ptr(out))
    return out.reshape(4, 4)


def mat4_vec4(M, v):
    out = np.zeros(4, np.float32)
    _lib.orc_mat4_vec4(_ptr(_f32(M, (16,))), _ptr(_f32(v, (4,))), _ptr(out))
    return out


def threads() -> int:
    return _lib.orc_threads()


class MethodGrid64:
    """FP64 oracle of the per-frame method (FP64 TSDF, trilinear raycast)."""

    def __init__(self, vl, trunc, resi, resj, intr=(525.0, 525.0, 319.5, 239.5), max_weight=0.0,
                 round_pixel=True):
        self.resi, self.resj, self.intr = resi, resj, intr
        self._h = _lib.orm_grid_new(vl, trunc, resi, resj, *map(float, intr), float(max_weight))
        _lib.orm_grid_set_round_pixel(self._h, 1 if round_pixel else 0)

    def __del__(self):
        if getattr(self, "_h", None):
            _lib.orm_grid_free(self._h)
            self._h = None

    def fuse(self, depth, T, deint=False) -> int:
        depth = np.ascontiguousarray(depth, np.uint16)
        T = np.ascontiguousarray(T, np.float64)
        return _lib.orm_grid_fuse(self._h, _ptr(depth), _ptr(T), int(deint))

    def count(self) -> int:
        return _lib.orm_grid_count(self._h)

    def import_blocks(self, coords, sdf, w):
        coords = np.ascontiguousarray(coords, np.int32)
        _lib.orm_grid_import(self._h, len(coords), _ptr(coords), _ptr(_f32(sdf)), _ptr(_f32(w)))

    def add_voxel(self, coords, v, delta) -> bool:
        return bool(_lib.orm_grid_add_voxel(self._h, int(coords[0]), int(coords[1]), int(coords[2]), int(v),
                                            float(delta)))

    def raycast_loss(self, T, obs, lambda_n=1.0, r_max=0.05, max_steps=128, t_min=0.2, t_max=10.0):
        valid = np.zeros(1, np.int64)
        obs = np.ascontiguousarray(obs, np.uint16)
        loss = _lib.orm_raycast_loss(self._h, _ptr(np.ascontiguousarray(T, np.float64)), _ptr(obs),
                                     float(lambda_n), float(r_max), int(max_steps), float(t_min), float(t_max),
                                     _ptr(valid))
        return loss, int(valid[0])

    def raycast_loss_pixels(self, T, obs, lambda_n=1.0, r_max=0.05, max_steps=128, t_min=0.2, t_max=10.0):
        """(per-pixel loss terms, per-pixel hit depths t*), [rows, cols] each, NaN where a pixel is not valid."""
        out = np.zeros((self.resi, self.resj))
        hit = np.zeros((self.resi, self.resj))
        obs = np.ascontiguousarray(obs, np.uint16)
        _lib.orm_raycast_loss_pixels(self._h, _ptr(np.ascontiguousarray(T, np.float64)), _ptr(obs), float(lambda_n),
                                     float(r_max), int(max_steps), float(t_min), float(t_max), C.c_void_p(), _ptr(out),
                                     _ptr(hit))
        return out, hit

    def raycast_loss_grad(self, T, obs, lambda_n=1.0, r_max=0.05, max_steps=128, t_min=0.2, t_max=10.0,
                          voxels=False):
        """(loss, dL/dxi [6]) or, with voxels=True, (loss, dL/dxi, dL/ds [blocks, 512] in export order)."""
        grad = np.zeros(6)
        gvox = np.zeros((self.count(), 512)) if voxels else None
        obs = np.ascontiguousarray(obs, np.uint16)
        loss = _lib.orm_raycast_loss_grad(self._h, _ptr(np.ascontiguousarray(T, np.float64)), _ptr(obs),
                                          float(lambda_n), float(r_max), int(max_steps), float(t_min), float(t_max),
                                          _ptr(grad), _ptr(gvox))
        return (loss, grad, gvox) if voxels else (loss, grad)

    def extract_mesh(self, method: str = "tetrahedra") -> np.ndarray:
        """Triangle soup [n, 3, 3] (FP64) by marching tetrahedra or marching cubes."""
        fn = _lib.orm_extract_mesh_cubes if method == "cubes" else _lib.orm_extract_mesh
        n = fn(self._h, 0, C.c_void_p())
        out = np.zeros((max(n, 1), 3, 3))
        fn(self._h, n, _ptr(out))
        return out[:n]

    def export(self) -> dict:
        n = self.count()
        keys = np.zeros(n, np.uint64)
        coords = np.zeros((n, 3), np.int32)
        sdf = np.zeros((n, 512), np.float64)
        w = np.zeros((n, 512), np.float64)
        _lib.orm_grid_export(self._h, n, _ptr(keys), _ptr(coords), _ptr(sdf), _ptr(w))
        return dict(keys=keys, coords=coords, sdf=sdf, w=w)

    def raycast(self, T, max_steps=128, t_min=0.2, t_max=10.0, hint=None, hint_margin=0.0):
        vmap = np.zeros((self.resi, self.resj, 4), np.float64)
        nmap = np.zeros((self.resi, self.resj, 4), np.float64)
        steps = np.zeros((self.resi, self.resj), np.int32)
        hint = np.ascontiguousarray(hint, np.uint16) if hint is not None else None
        _lib.orm_raycast(self._h, _ptr(np.ascontiguousarray(T, np.float64)), int(max_steps), float(t_min),
                         float(t_max), _ptr(hint), float(hint_margin), _ptr(vmap), _ptr(nmap), _ptr(steps))
        return vmap, nmap, steps


def track64(depth, vmap, nmap, Tprev, T0, intr=(525.0, 525.0, 319.5, 239.5), levels=3, iters=(10, 5, 4),
            dist=(0.06, 0.10, 0.15), rmin=0.2, dmax=10.0):
    """FP64 frame-to-model point-to-plane Gauss-Newton (the method of the GPU tracker)."""
    depth = np.ascontiguousarray(depth, np.uint16)
    rows, cols = depth.shape
    T = np.ascontiguousarray(T0, np.float64).copy()
    it = np.ascontiguousarray(list(iters) + [0] * (4 - len(iters)), np.int32)
    ds = np.ascontiguousarray(list(dist) + [0.2] * (4 - len(dist)), np.float64)
    n = _lib.orm_track(_ptr(depth), rows, cols, *map(float, intr), _ptr(np.ascontiguousarray(vmap, np.float64)),
                       _ptr(np.ascontiguousarray(nmap, np.float64)), _ptr(np.ascontiguousarray(Tprev, np.float64)),
                       _ptr(T), int(levels), _ptr(it), _ptr(ds), float(rmin), float(dmax))
    return T, n


# ---- integration scheduling (src/core/integrate.cpp:47-236), numpy restatement ----

def dofs_to_pose(x):
    """getT (src/utils/matrixutil.h:61-63): trans(x[3:6]) @ Rz(x[2]) @ Ry(x[1]) @ Rx(x[0]), as the product."""
    x = np.asarray(x, np.float64)
    def rx(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[1, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, 1.0]])
    def ry(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[c, 0, s, 0], [0, 1, 0, 0], [-s, 0, c, 0], [0, 0, 0, 1.0]])
    def rz(a):
        c, s = np.cos(a), np.sin(a)
        return np.array([[c, -s, 0, 0], [s, c, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1.0]])
    t = np.eye(4)
    t[:3, 3] = x[3:6]
    return t @ rz(x[2]) @ ry(x[1]) @ rx(x[0])


def pose_to_dofs(T):
    """MattoDof (src/utils/matrixutil.cpp:37-49)."""
    T = np.asarray(T, np.float64)
    return np.array([np.arctan2(T[2, 1], T[2, 2]), -np.arcsin(T[2, 0]), np.arctan2(T[1, 0], T[0, 0]),
                     T[0, 3], T[1, 3], T[2, 3]])


def pose_change(world, integrated):
    """diff (src/core/integrate.cpp:205-211): |(d rotation DoFs, 2 d translation DoFs)|."""
    d = np.asarray(world, np.float64) - np.asarray(integrated, np.float64)
    s = 0.0
    for k in range(6):  # squared norm summed in element order
        v = (1.0 if k < 3 else 2.0) * float(d[k])
        s += v * v
    return float(np.sqrt(s))


def reintegration_order(world, integrated, treint):
    """updateReintegrationBuffer (integrate.cpp:218-236): stable sort by descending
    diff (std::list::sort), then the prefix with diff >= treint."""
    d = [pose_change(w, i) for w, i in zip(world, integrated)]
    idx = sorted(range(len(d)), key=lambda k: -d[k])  # Python's sort is stable
    out = []
    for k in idx:
        if d[k] < treint:
            break
        out.append(k)
    return out
