"""ctypes binding of libkinfu_gb300.so (the C ABI declared in include/kinfu_gb300.h).

The shared library is the product: every compute call below goes to the CUDA
kernels in it.  There is no CPU fallback -- if the library is missing or no CUDA
device is usable, calls fail with an error.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = Path(os.environ.get("KINFU_GB300_LIB", PKG / "lib" / "libkinfu_gb300.so"))
HEADER = PKG.parent / "include" / "kinfu_gb300.h"

KF_OK = 0
KF_ERR_INVALID_ARGUMENT = 1
KF_ERR_CUDA = 2
KF_ERR_OUT_OF_MEMORY = 3
KF_ERR_STATE = 4
KF_ERR_IO = 5
KF_ERR_UNSUPPORTED = 6

KF_TSDF_F32 = 0
KF_TSDF_F16 = 1
KF_ICP_FAIL_REFERENCE = 0
KF_ICP_FAIL_IDENTITY = 1
KF_REDUCE_REFERENCE_ORDER = 0
KF_REDUCE_TREE = 1
KF_SOLVE_REFERENCE = 0
KF_SOLVE_PRECISE = 1


class KinfuError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"kinfu_gb300 status {status}: {message}")
        self.status = status


class Config(C.Structure):
    """kf_config (include/kinfu_gb300.h)."""

    _fields_ = [
        ("height", C.c_int),
        ("width", C.c_int),
        ("min_depth", C.c_float),
        ("max_depth", C.c_float),
        ("dims", C.c_int * 3),
        ("grid_start", C.c_int * 3),
        ("voxel_size", C.c_float),
        ("truncated_distance", C.c_float),
        ("sdf_minimum", C.c_float),
        ("sdf_maximum", C.c_float),
        ("icp_levels", C.c_int),
        ("icp_iterations", C.c_int * 3),
        ("icp_distance", C.c_float),
        ("icp_angle_deg", C.c_float),
        ("icp_fail_mode", C.c_int),
        ("icp_reduction", C.c_int),
        ("solve_mode", C.c_int),
        ("tsdf_storage", C.c_int),
        ("bilateral", C.c_int),
        ("bilateral_radius", C.c_int),
        ("sigma_d", C.c_float),
        ("sigma_r", C.c_float),
        ("use_graphs", C.c_int),
    ]


class RenderDesc(C.Structure):
    """kf_render_desc (include/kinfu_gb300.h): the differentiation form's camera and grid."""

    _fields_ = [("height", C.c_int), ("width", C.c_int), ("fx", C.c_float), ("fy", C.c_float), ("cx", C.c_float),
                ("cy", C.c_float), ("dims", C.c_int * 3), ("grid_start", C.c_int * 3), ("voxel_size", C.c_float),
                ("t_near", C.c_float), ("t_far", C.c_float), ("step", C.c_float)]


_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_H = C.c_void_p  # kf_handle*

# name -> (restype, argtypes); mirrors include/kinfu_gb300.h
SIGNATURES = {
    "kf_config_default": (None, [C.POINTER(Config)]),
    "kf_create": (C.c_int, [C.POINTER(Config), C.POINTER(_H)]),
    "kf_destroy": (C.c_int, [_H]),
    "kf_last_error": (C.c_char_p, [_H]),
    "kf_status_string": (C.c_char_p, [C.c_int]),
    "kf_get_config": (C.c_int, [_H, C.POINTER(Config)]),
    "kf_set_intrinsics": (C.c_int, [_H, C.c_float, C.c_float, C.c_float, C.c_float]),
    "kf_set_intrinsics_ex": (C.c_int, [_H, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int]),
    "kf_get_intrinsics": (C.c_int, [_H, _f32p]),
    "kf_set_pose": (C.c_int, [_H, _f32p]),
    "kf_get_pose": (C.c_int, [_H, _f32p]),
    "kf_reset": (C.c_int, [_H]),
    "kf_initial_processing": (C.c_int, [_H, _vp]),
    "kf_incoming_frame": (C.c_int, [_H, _vp]),
    "kf_process_frame": (C.c_int, [_H, _vp, C.c_int]),
    "kf_initial_processing_device": (C.c_int, [_H, _vp]),
    "kf_incoming_frame_device": (C.c_int, [_H, _vp]),
    "kf_load_depth_dat": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, _u16p]),
    "kf_synchronize": (C.c_int, [_H]),
    "kf_set_stream": (C.c_int, [_H, _vp]),
    "kf_get_predicted": (C.c_int, [_H, _vp, _vp, _vp, _vp, _vp, _vp]),
    "kf_get_volume": (C.c_int, [_H, _vp, _vp]),
    "kf_set_volume": (C.c_int, [_H, _f32p, _f32p]),
    "kf_get_depth": (C.c_int, [_H, _f32p]),
    "kf_get_icp_stats": (C.c_int, [_H, _vp, _vp, _vp, C.c_int]),
    "kf_set_depth_f32": (C.c_int, [_H, _f32p]),
    "kf_set_depth_u16": (C.c_int, [_H, _u16p]),
    "kf_calculate_vertices_and_normals": (C.c_int, [_H, _vp, _vp, _vp, _vp, _vp, _vp]),
    "kf_bilateral_filtering": (C.c_int, [_H]),
    "kf_estimate_sensor_pose": (C.c_int, [_H]),
    "kf_projective_tsdf": (C.c_int, [_H, C.c_int]),
    "kf_ray_casting": (C.c_int, [_H, _vp]),
    "kf_set_predicted": (C.c_int, [_H, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p]),
    "kf_icp_associate": (C.c_int, [_H, _f32p, _f32p, _vp, _vp, _vp]),
    "kf_get_flip_threshold": (C.c_int, [_H, C.POINTER(C.c_float)]),
    "kf_enable_stage_timing": (C.c_int, [_H, C.c_int]),
    "kf_get_stage_times": (C.c_int, [_H, _f32p]),
    "kf_kernels_per_frame": (C.c_int, [_H, C.POINTER(C.c_int)]),
    "kf_set_wait_limit": (C.c_int, [_H, C.c_longlong]),
    "kf_export_ply": (C.c_int, [_H, C.c_char_p, C.c_void_p, C.POINTER(C.c_int)]),
    "kf_save_checkpoint": (C.c_int, [_H, C.c_char_p]),
    "kf_load_checkpoint": (C.c_int, [_H, C.c_char_p]),
    "kf_render_trilinear": (C.c_int, [C.POINTER(RenderDesc), C.c_void_p, _f32p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "kf_render_trilinear_backward": (C.c_int, [C.POINTER(RenderDesc), C.c_void_p, _f32p, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p, C.c_void_p]),
    "kf_render_depth_normal_equations": (C.c_int, [C.POINTER(RenderDesc), C.c_void_p, _f32p, C.c_void_p, C.c_float,
                                                   C.POINTER(C.c_double), C.c_void_p]),
    "kf_render_depth_normal_equations_huber": (C.c_int, [C.POINTER(RenderDesc), C.c_void_p, _f32p, C.c_void_p,
                                                         C.c_float, C.c_float, C.POINTER(C.c_double), C.c_void_p]),
    "kf_batch_create": (C.c_int, [C.POINTER(Config), C.c_int, C.POINTER(C.c_void_p)]),
    "kf_batch_destroy": (C.c_int, [C.c_void_p]),
    "kf_batch_scene": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(_H)]),
    "kf_batch_initial_processing_device": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "kf_batch_incoming_frame_device": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "kf_batch_synchronize": (C.c_int, [C.c_void_p]),
    "kf_batch_kernels_per_frame": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "kf_batch_autotune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "kf_batch_set_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "kf_batch_set_forms": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "kf_selftest_solve": (C.c_int, [C.c_ulonglong, C.c_int, C.c_int, C.POINTER(C.c_ulonglong)]),
    "kf_selftest_solve6": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    "kf_icp_associate_noalloc": (C.c_int, [C.c_int, C.c_int, _f32p, _f32p, _f32p, _vp, _vp, _vp, _vp, C.c_float,
                                           C.c_float, _vp, _vp, _vp]),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load (once) and return the library; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the kinfu_gb300 library has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def declared_symbols(header: Path = HEADER) -> list[str]:
    """Every kf_* function the public header declares."""
    import re

    text = header.read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(kf_\w+)\s*\(", text, re.M)))


def default_config() -> Config:
    cfg = Config()
    load().kf_config_default(C.byref(cfg))
    return cfg


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(C.c_void_p)
