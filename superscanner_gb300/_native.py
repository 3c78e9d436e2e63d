"""ctypes binding of libss.so (the C-ABI declared in include/ss_abi.h)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libss.so"

if not LIB_PATH.exists():
    raise ImportError(
        f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
        "(there is no CPU fallback for the reconstruction path)")

lib = C.CDLL(str(LIB_PATH))

STATUS = {
    0: "SS_OK", 1: "SS_ERR_ARG", 2: "SS_ERR_DIMS", 3: "SS_ERR_TABLE_FULL", 4: "SS_ERR_LIST_OVERFLOW",
    5: "SS_ERR_TIMEOUT", 6: "SS_ERR_CUDA", 7: "SS_ERR_RANGE", 8: "SS_ERR_STATE", 9: "SS_ERR_NOMEM",
}
SS_OK, SS_ERR_ARG, SS_ERR_DIMS, SS_ERR_TABLE_FULL, SS_ERR_LIST_OVERFLOW = 0, 1, 2, 3, 4
SS_ERR_TIMEOUT, SS_ERR_CUDA, SS_ERR_RANGE, SS_ERR_STATE, SS_ERR_NOMEM = 5, 6, 7, 8, 9
SS_STORAGE_F32, SS_STORAGE_F16 = 0, 1


class SSError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        detail = lib.ss_last_error().decode(errors="replace") if code == SS_ERR_CUDA else ""
        super().__init__(f"{where}: {STATUS.get(code, code)} {detail}".strip())


def check(code: int, where: str) -> int:
    if code != SS_OK:
        raise SSError(code, where)
    return code


class SSParams(C.Structure):
    _fields_ = [
        ("voxel_length", C.c_float), ("truncation", C.c_float), ("resi", C.c_int32), ("resj", C.c_int32),
        ("hash_buckets", C.c_uint32), ("storage", C.c_int32), ("with_color", C.c_int32),
        ("max_weight", C.c_float), ("rmin", C.c_float), ("d_max", C.c_float),
    ]


_p, _i32, _u32, _f, _st = C.c_void_p, C.c_int32, C.c_uint32, C.c_float, C.c_int
_F16 = C.POINTER(C.c_float)
_D16 = C.POINTER(C.c_double)

class SSLaunchConfig(C.Structure):
    _fields_ = [("collect_rows", C.c_int32), ("raycast_rows", C.c_int32), ("fuse_ctas_per_sm", C.c_int32),
                ("refuse_ctas_per_sm", C.c_int32), ("track_ctas_per_sm", C.c_int32)]


class SSPipelineParams(C.Structure):
    _fields_ = [
        ("levels", C.c_int32), ("iters", C.c_int32 * 4), ("dist_thresh", C.c_float * 4),
        ("raycast_steps", C.c_int32), ("t_min", C.c_float), ("t_max", C.c_float),
        ("use_graph", C.c_int32), ("exact_fusion", C.c_int32), ("hint_margin", C.c_float),
        ("persistent_track", C.c_int32),
    ]


# name: (restype, argtypes); every symbol the header declares is listed here
# and checked by tests/test_abi.py.
SIGNATURES = {
    "ss_last_error": (C.c_char_p, []),
    "ss_params_default": (_st, [C.POINTER(SSParams), _u32, _f, _f, _i32, _i32]),
    "ss_grid_create": (_st, [C.POINTER(SSParams), C.POINTER(_p)]),
    "ss_grid_destroy": (_st, [_p]),
    "ss_grid_reset": (_st, [_p, _p]),
    "ss_grid_get_launch_config": (_st, [_p, C.POINTER(SSLaunchConfig)]),
    "ss_grid_set_launch_config": (_st, [_p, C.POINTER(SSLaunchConfig)]),
    "ss_grid_set_intrinsic": (_st, [_p, _f, _f, _f, _f]),
    "ss_integrate": (_st, [_p, _p, _p, _F16, _i32, _p]),
    "ss_deintegrate": (_st, [_p, _p, _p, _F16, _i32, _p]),
    "ss_integrate_fast": (_st, [_p, _p, _p, _F16, _i32, _i32, _p]),
    "ss_raycast": (_st, [_p, _F16, _p, _p, _p]),
    "ss_clean_memory": (_st, [_p, _p]),
    "ss_refuse_batch": (_st, [_p, _i32, _p, _p, _p, _i32, _p]),
    "ss_grid_extract_mesh": (_st, [_p, C.c_int64, _p, C.POINTER(C.c_int64), _p]),
    "ss_grid_extract_mesh_cubes": (_st, [_p, C.c_int64, _p, C.POINTER(C.c_int64), _p]),
    "ss_png_unfilter": (_st, [_p, _i32, _i32, _i32, _p]),
    "ss_jpeg_create": (_st, [C.POINTER(_p)]),
    "ss_jpeg_destroy": (_st, [_p]),
    "ss_jpeg_info": (_st, [_p, _p, C.c_size_t, C.POINTER(_i32), C.POINTER(_i32)]),
    "ss_jpeg_decode_rgb": (_st, [_p, _p, C.c_size_t, _p, _i32, _i32, _p]),
    "ss_resize_rgb": (_st, [_p, _i32, _i32, _p, _i32, _i32, _p]),
    "ss_dofs_to_pose": (_st, [_D16, _D16]),
    "ss_pose_to_dofs": (_st, [_D16, _D16]),
    "ss_reintegration_order": (_st, [_i32, _p, _p, C.c_double, _p, C.POINTER(_i32)]),
    "ss_scheduler_create": (_st, [_p, C.c_double, _i32, _i32, _p]),
    "ss_scheduler_destroy": (_st, [_p]),
    "ss_scheduler_push_integrate": (_st, [_p, C.c_int64, _p, _D16]),
    "ss_scheduler_set_dofs": (_st, [_p, C.c_int64, _D16]),
    "ss_scheduler_push_deintegrate": (_st, [_p, C.c_int64]),
    "ss_scheduler_update": (_st, [_p, C.POINTER(_i32)]),
    "ss_scheduler_queue": (_st, [_p, _i32, _i32, _p, C.POINTER(_i32)]),
    "ss_scheduler_step": (_st, [_p, _p, C.POINTER(_i32)]),
    "ss_scheduler_drain": (_st, [_p, _p, C.POINTER(_i32)]),
    "ss_scheduler_frame": (_st, [_p, C.c_int64, C.POINTER(_i32), _D16]),
    "ss_grid_sync": (_st, [_p, _p]),
    "ss_grid_block_count": (_st, [_p, _p, C.POINTER(_i32)]),
    "ss_grid_counters": (_st, [_p, _p, C.POINTER(C.c_int64)]),
    "ss_grid_raycast_counters": (_st, [_p, _p, C.POINTER(C.c_int64)]),
    "ss_grid_test_raycast_cap": (_st, [_p, C.c_int32]),
    "ss_test_fixed48_sum": (_st, [_p, _i32, C.POINTER(C.c_double), _p]),
    "ss_pipeline_test_wait_timeout": (_st, [_p, C.c_int32]),
    "ss_grid_export_blocks": (_st, [_p, _p, _i32, _p, _p, _p, _p, _p, C.POINTER(_i32)]),
    "ss_grid_export_buckets": (_st, [_p, _p, _i32, _p, C.POINTER(_i32)]),
    "ss_grid_import_blocks": (_st, [_p, _p, _i32, _p, _p, _p, _p]),
    "ss_depth_to_pcd": (_st, [_p, _i32, _i32, _f, _f, _f, _f, _p, _p]),
    "ss_normals_from_pcd": (_st, [_p, _i32, _i32, _p, _p]),
    "ss_kokkos_icp": (_st, [_p, _p, _i32, _i32, _f, _f, _f, _f, _D16, _D16, _i32, _D16,
                            C.POINTER(C.c_float), _p]),
    "ss_kokkos_icp_noalloc": (_st, [_p, _p, _i32, _i32, _f, _f, _f, _f, _D16, _D16, _i32, _D16,
                                    C.POINTER(C.c_float), _p]),
    "ss_raycast_maps": (_st, [_p, _F16, _i32, _f, _f, _p, _f, _p, _p, _p]),
    "ss_raycast_loss": (_st, [_p, _D16, _p, _f, _f, _i32, C.POINTER(C.c_double), C.POINTER(C.c_int64), _p, _p]),
    "ss_raycast_loss_grad": (_st, [_p, _D16, _p, _f, _f, _i32, C.POINTER(C.c_double), C.POINTER(C.c_double), _p,
                                   C.POINTER(C.c_int64), _p]),
    "ss_raycast_loss_grad_masked": (_st, [_p, _D16, _p, _p, _f, _f, _i32, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), _p, C.POINTER(C.c_int64), _p]),
    "ss_pipeline_params_default": (_st, [C.POINTER(SSPipelineParams)]),
    "ss_pipeline_create": (_st, [_p, C.POINTER(SSPipelineParams), C.POINTER(_p)]),
    "ss_pipeline_destroy": (_st, [_p]),
    "ss_pipeline_set_pose": (_st, [_p, _D16, _p]),
    "ss_pipeline_get_pose": (_st, [_p, _D16, _p]),
    "ss_pipeline_set_start": (_st, [_p, _D16, _p]),
    "ss_pipeline_input": (_st, [_p, C.POINTER(_p)]),
    "ss_pipeline_read_pose": (_st, [_p, _p, _p]),
    "ss_pipeline_maps": (_st, [_p, C.POINTER(_p), C.POINTER(_p)]),
    "ss_pipeline_frame": (_st, [_p, _p, _i32, _p]),
    "ss_pipeline_stats": (_st, [_p, C.POINTER(_i32), C.POINTER(_f), _p]),
    "ss_pipeline_copy_maps": (_st, [_p, _p, _p, _p]),
    "ss_pipeline_profile": (_st, [_p, _i32]),
    "ss_pipeline_stage_ms": (_st, [_p, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int64), _p]),
}

for _name, (_res, _args) in SIGNATURES.items():
    _fn = getattr(lib, _name)
    _fn.restype = _res
    _fn.argtypes = _args


def f32x16(m) -> C.Array:
    import numpy as np
    a = np.ascontiguousarray(np.asarray(m, dtype=np.float32).reshape(16))
    return (C.c_float * 16)(*a.tolist())


def f64x16(m) -> C.Array:
    import numpy as np
    a = np.ascontiguousarray(np.asarray(m, dtype=np.float64).reshape(16))
    return (C.c_double * 16)(*a.tolist())
