"""kinect_fusion_slam_gb300 -- GB300-native KinectFusion per-frame path.

Python host side of the kinfu_gb300 C ABI (include/kinfu_gb300.h).  ``KinfuPipeline``
mirrors the reference's ``Kinfu::KinfuPipeline`` (src/kinfu_pipeline.h:11-68):
constructor ``(height, width, max_depth, min_depth)``, ``intrinsic_matrix`` and
``extrinsic_matrix`` (4x4 row-major camera-to-world, mm), ``InitialProcessing`` /
``IncomingFrameProcessing``, ``global_tsdf`` / ``global_weight_tsdf`` in the
reference's z-fastest order, and the surface-prediction planes read by its viewer
(system_utility.h:26-35).  ``Handle`` exposes every C entry point, including the
five stage launchers of src/parallel_processing/parallel_processing.h:19-53.

All compute runs in the CUDA library; nothing here falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import (KF_ERR_CUDA, KF_ERR_INVALID_ARGUMENT, KF_ERR_IO, KF_ERR_OUT_OF_MEMORY, KF_ERR_STATE,
                   KF_ERR_UNSUPPORTED, KF_ICP_FAIL_IDENTITY, KF_ICP_FAIL_REFERENCE, KF_OK, KF_REDUCE_REFERENCE_ORDER,
                   KF_REDUCE_TREE, KF_SOLVE_PRECISE, KF_SOLVE_REFERENCE, KF_TSDF_F16, KF_TSDF_F32, Config, KinfuError)

__all__ = ["KinfuPipeline", "Handle", "Batch", "Config", "KinfuError", "make_config", "KF_TSDF_F32", "KF_TSDF_F16",
           "KF_ICP_FAIL_REFERENCE", "KF_ICP_FAIL_IDENTITY", "KF_SOLVE_REFERENCE", "KF_SOLVE_PRECISE",
           "KF_REDUCE_REFERENCE_ORDER", "KF_REDUCE_TREE"]


def make_config(**kw) -> Config:
    """kf_config with the reference defaults, overridden by keyword (tuples for the
    array fields: dims, grid_start, icp_iterations)."""
    cfg = _lib.default_config()
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise KeyError(f"unknown kf_config field {k!r}")
        field = getattr(cfg, k)
        if isinstance(field, C.Array):
            vals = list(v)
            for i in range(len(field)):
                field[i] = vals[i] if i < len(vals) else 0
        else:
            setattr(cfg, k, v)
    return cfg


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


class Handle:
    """One kf_handle: device-resident volume, images, pose and stream."""

    def __init__(self, config: Config | None = None, **kw):
        self.lib = _lib.load()
        self.config = config if config is not None else make_config(**kw)
        h = _lib._H()
        st = self.lib.kf_create(C.byref(self.config), C.byref(h))
        if st != _lib.KF_OK:
            raise KinfuError(st, f"kf_create failed ({self.lib.kf_status_string(st).decode()})")
        self.h = h
        self.H, self.W = self.config.height, self.config.width
        self.dims = tuple(self.config.dims)

    # -- plumbing -----------------------------------------------------------------
    def _check(self, st: int) -> None:
        if st != _lib.KF_OK:
            raise KinfuError(st, self.lib.kf_last_error(self.h).decode())

    @classmethod
    def _borrowed(cls, ptr, config: Config, owner) -> "Handle":
        """A view of a handle owned elsewhere (a batch's scene); closing it does nothing."""
        self = cls.__new__(cls)
        self.lib = _lib.load()
        self.config = config
        self.h = ptr
        self.H, self.W = config.height, config.width
        self.dims = tuple(config.dims)
        self._owner = owner
        return self

    def close(self) -> None:
        if getattr(self, "_owner", None) is not None:
            self.h = None
            return
        if getattr(self, "h", None):
            self.lib.kf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def nvox(self) -> int:
        return int(self.dims[0]) * int(self.dims[1]) * int(self.dims[2])

    def _u16(self, depth) -> np.ndarray:
        d = np.ascontiguousarray(depth, dtype=np.uint16)
        if d.size != self.H * self.W:
            raise ValueError(f"depth must hold {self.H}x{self.W} values, got {d.shape}")
        return d

    # -- camera and pose ------------------------------------------------------------
    def set_intrinsics(self, fx, fy, cx, cy, one_based: bool = True) -> None:
        """fx, fy and the principal point: 1-based (the reference's K) unless one_based
        is False"""
        self._check(self.lib.kf_set_intrinsics_ex(self.h, fx, fy, cx, cy, int(one_based)))

    def intrinsics(self) -> np.ndarray:
        K = np.zeros(9, np.float32)
        self._check(self.lib.kf_get_intrinsics(self.h, K))
        return K.reshape(3, 3)

    def set_pose(self, T) -> None:
        self._check(self.lib.kf_set_pose(self.h, _f32(T).ravel()))

    def pose(self) -> np.ndarray:
        T = np.zeros(16, np.float32)
        self._check(self.lib.kf_get_pose(self.h, T))
        return T.reshape(4, 4)

    def reset(self) -> None:
        self._check(self.lib.kf_reset(self.h))

    # -- frame loop -----------------------------------------------------------------
    def initial_processing(self, depth_u16) -> None:
        d = self._u16(depth_u16)
        self._check(self.lib.kf_initial_processing(self.h, _lib.ptr(d)))

    def incoming_frame(self, depth_u16) -> None:
        d = self._u16(depth_u16)
        self._check(self.lib.kf_incoming_frame(self.h, _lib.ptr(d)))

    def process_frame(self, depth_u16, is_first: bool) -> None:
        """initial_processing when is_first, else incoming_frame (kf_process_frame)"""
        d = self._u16(depth_u16)
        self._check(self.lib.kf_process_frame(self.h, _lib.ptr(d), int(is_first)))

    def initial_processing_ptr(self, host_ptr: int) -> None:
        """host_ptr: address of H*W uint16 (pinned host memory avoids a staging copy)"""
        self._check(self.lib.kf_initial_processing(self.h, C.c_void_p(host_ptr)))

    def incoming_frame_ptr(self, host_ptr: int) -> None:
        self._check(self.lib.kf_incoming_frame(self.h, C.c_void_p(host_ptr)))

    def initial_processing_device(self, dev_ptr: int) -> None:
        self._check(self.lib.kf_initial_processing_device(self.h, C.c_void_p(dev_ptr)))

    def incoming_frame_device(self, dev_ptr: int) -> None:
        self._check(self.lib.kf_incoming_frame_device(self.h, C.c_void_p(dev_ptr)))

    def set_stream(self, stream_handle: int | None) -> None:
        """Run on a caller-owned cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self.lib.kf_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None))

    def synchronize(self) -> None:
        self._check(self.lib.kf_synchronize(self.h))

    # -- readback ---------------------------------------------------------------------
    def predicted(self) -> np.ndarray:
        """(6, H, W): surface_prediction_{x,y,z}, surface_prediction_normal_{x,y,z}"""
        out = np.zeros((6, self.H, self.W), np.float32)
        self._check(self.lib.kf_get_predicted(self.h, *[_lib.ptr(out[k]) for k in range(6)]))
        return out

    def export_ply(self, path, colour_bgr=None) -> int:
        """Write the latest predicted surface as a binary PLY (the viewer's point cloud);
        colour_bgr: optional (H, W, 3) uint8 BGR image.  Returns the point count."""
        n = C.c_int(0)
        col = None
        if colour_bgr is not None:
            col = np.ascontiguousarray(colour_bgr, np.uint8)
            if col.shape != (self.H, self.W, 3):
                raise ValueError(f"colour image must be ({self.H}, {self.W}, 3)")
        self._check(self.lib.kf_export_ply(self.h, str(path).encode(), _lib.ptr(col), C.byref(n)))
        return int(n.value)

    def save_checkpoint(self, path) -> None:
        self._check(self.lib.kf_save_checkpoint(self.h, str(path).encode()))

    def load_checkpoint(self, path) -> None:
        self._check(self.lib.kf_load_checkpoint(self.h, str(path).encode()))

    def set_predicted(self, pred6) -> None:
        p = _f32(pred6).reshape(6, self.H, self.W)
        self._check(self.lib.kf_set_predicted(self.h, *[np.ascontiguousarray(p[k]).ravel() for k in range(6)]))

    def volume(self, tsdf: bool = True, weight: bool = True):
        t = np.empty(self.nvox, np.float32) if tsdf else None
        w = np.empty(self.nvox, np.float32) if weight else None
        self._check(self.lib.kf_get_volume(self.h, _lib.ptr(t), _lib.ptr(w)))
        return t, w

    def set_volume(self, tsdf, weight) -> None:
        self._check(self.lib.kf_set_volume(self.h, _f32(tsdf).ravel(), _f32(weight).ravel()))

    def depth(self) -> np.ndarray:
        d = np.zeros((self.H, self.W), np.float32)
        self._check(self.lib.kf_get_depth(self.h, d.ravel()))
        return d

    def icp_stats(self, n: int | None = None, poses: bool = False):
        """Per-iteration correspondences and Cholesky success of the latest ICP (and the
        pose after each iteration when poses=True)."""
        n = n or int(sum(self.config.icp_iterations[:max(1, int(self.config.icp_levels))]))
        nc = np.zeros(n, np.int32)
        ok = np.zeros(n, np.int32)
        Ts = np.zeros((n, 4, 4), np.float32) if poses else None
        self._check(self.lib.kf_get_icp_stats(self.h, _lib.ptr(nc), _lib.ptr(ok), _lib.ptr(Ts), n))
        return (nc, ok, Ts) if poses else (nc, ok)

    # -- stage launchers (parallel_processing.h:19-53) --------------------------------
    def set_depth_f32(self, depth) -> None:
        self._check(self.lib.kf_set_depth_f32(self.h, _f32(depth).ravel()))

    def set_depth_u16(self, depth) -> None:
        self._check(self.lib.kf_set_depth_u16(self.h, self._u16(depth).ravel()))

    def calculate_vertices_and_normals(self):
        out = np.zeros((5, self.H, self.W), np.float32)
        mask = np.zeros((self.H, self.W), np.uint8)
        self._check(self.lib.kf_calculate_vertices_and_normals(self.h, *[_lib.ptr(out[k]) for k in range(5)],
                                                               _lib.ptr(mask)))
        return out, mask

    def bilateral_filtering(self) -> None:
        self._check(self.lib.kf_bilateral_filtering(self.h))

    def estimate_sensor_pose(self) -> np.ndarray:
        self._check(self.lib.kf_estimate_sensor_pose(self.h))
        return self.pose()

    def projective_tsdf(self, first: bool) -> None:
        self._check(self.lib.kf_projective_tsdf(self.h, 1 if first else 0))

    def ray_casting(self) -> np.ndarray:
        hit = np.zeros((self.H, self.W), np.int32)
        self._check(self.lib.kf_ray_casting(self.h, _lib.ptr(hit)))
        return hit

    def icp_associate(self, F, T):
        pair = np.zeros((self.H, self.W), np.int32)
        sums = np.zeros(27, np.float32)
        n = C.c_int32(0)
        self._check(self.lib.kf_icp_associate(self.h, _f32(F).ravel(), _f32(T).ravel(), _lib.ptr(pair),
                                              _lib.ptr(sums), C.cast(C.pointer(n), C.c_void_p)))
        return int(n.value), sums, pair

    def flip_threshold(self) -> float:
        c = C.c_float(0)
        self._check(self.lib.kf_get_flip_threshold(self.h, C.byref(c)))
        return c.value

    # -- timing ---------------------------------------------------------------------
    def enable_stage_timing(self, on: bool = True) -> None:
        self._check(self.lib.kf_enable_stage_timing(self.h, 1 if on else 0))

    def stage_times(self) -> np.ndarray:
        ms = np.zeros(5, np.float32)
        self._check(self.lib.kf_get_stage_times(self.h, ms))
        return ms

    def set_wait_limit(self, polls: int) -> None:
        """Poll limit of the bounded device waits (kf_set_wait_limit): 0 makes every
        bounded wait give up at once, a negative value restores the default."""
        self._check(self.lib.kf_set_wait_limit(self.h, int(polls)))

    def kernels_per_frame(self) -> int:
        n = C.c_int(0)
        self._check(self.lib.kf_kernels_per_frame(self.h, C.byref(n)))
        return n.value


def load_depth_dat(data_dir, frame_index: int, height: int = 480, width: int = 640) -> np.ndarray:
    """SystemUtility::LoadDepthData's file read (system_utility.cpp:58-68)."""
    out = np.zeros((height, width), np.uint16)
    st = _lib.load().kf_load_depth_dat(str(data_dir).encode(), frame_index, height, width, out.ravel())
    if st != _lib.KF_OK:
        raise KinfuError(st, f"cannot read {data_dir}/dep{frame_index:04d}.dat")
    return out


class KinfuPipeline:
    """Kinfu::KinfuPipeline (src/kinfu_pipeline.h:11-68) over the GB300 library.

    ``InitialProcessing(frame)`` / ``IncomingFrameProcessing(frame, per_nth_frame)``
    accept either a frame index (read as ``<data_dir>/dep%04d.dat``, the reference's
    ``../data``) or an (H, W) uint16 depth array."""

    def __init__(self, height: int = 480, width: int = 640, max_depth: float = 2000.0, min_depth: float = 300.0,
                 data_dir: str | os.PathLike = "../data", **config):
        self.handle = Handle(make_config(height=height, width=width, max_depth=max_depth, min_depth=min_depth,
                                         **config))
        self.data_dir = Path(data_dir)
        self.height, self.width = height, width

    # reference members
    @property
    def intrinsic_matrix(self) -> np.ndarray:
        return self.handle.intrinsics()

    @intrinsic_matrix.setter
    def intrinsic_matrix(self, K) -> None:
        K = np.asarray(K, np.float64)
        self.handle.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])

    @property
    def extrinsic_matrix(self) -> np.ndarray:
        return self.handle.pose()

    @extrinsic_matrix.setter
    def extrinsic_matrix(self, T) -> None:
        self.handle.set_pose(T)

    @property
    def global_tsdf(self) -> np.ndarray:
        return self.handle.volume(weight=False)[0]

    @property
    def global_weight_tsdf(self) -> np.ndarray:
        return self.handle.volume(tsdf=False)[1]

    def _depth(self, frame) -> np.ndarray:
        if isinstance(frame, (int, np.integer)):
            return load_depth_dat(self.data_dir, int(frame), self.height, self.width)
        return frame

    def InitialProcessing(self, start_frame) -> None:
        self.handle.initial_processing(self._depth(start_frame))

    def IncomingFrameProcessing(self, current_frame, per_nth_frame: int = 1) -> None:
        # per_nth_frame is accepted for interface parity; the reference ignores it too
        self.handle.incoming_frame(self._depth(current_frame))

    def surface_prediction(self) -> dict:
        p = self.handle.predicted()
        keys = ["surface_prediction_x", "surface_prediction_y", "surface_prediction_z",
                "surface_prediction_normal_x", "surface_prediction_normal_y", "surface_prediction_normal_z"]
        return dict(zip(keys, p))

    def close(self) -> None:
        self.handle.close()


class Batch:
    """The batching form (kf_batch_*): independent scenes of uneven image and grid
    sizes, every stage one launch for all of them, each frame one CUDA graph."""

    def __init__(self, configs):
        self.lib = _lib.load()
        self.configs = list(configs)
        arr = (Config * len(self.configs))(*self.configs)
        b = C.c_void_p()
        st = self.lib.kf_batch_create(arr, len(self.configs), C.byref(b))
        if st != _lib.KF_OK:
            raise KinfuError(st, "kf_batch_create failed")
        self.b = b
        self.scenes = []
        for i, cfg in enumerate(self.configs):
            h = _lib._H()
            self._check(self.lib.kf_batch_scene(self.b, i, C.byref(h)))
            self.scenes.append(Handle._borrowed(h, cfg, self))

    def _check(self, st: int) -> None:
        if st != _lib.KF_OK:
            raise KinfuError(st, "kf_batch call failed")

    def close(self) -> None:
        if getattr(self, "b", None):
            for h in self.scenes:
                h.h = None
            self.lib.kf_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ptrs(self, dev_ptrs):
        if len(dev_ptrs) != len(self.scenes):
            raise ValueError("one depth pointer per scene")
        return (C.c_void_p * len(dev_ptrs))(*[C.c_void_p(int(p)) for p in dev_ptrs])

    def initial_processing_device(self, dev_ptrs) -> None:
        self._check(self.lib.kf_batch_initial_processing_device(self.b, self._ptrs(dev_ptrs)))

    def incoming_frame_device(self, dev_ptrs) -> None:
        self._check(self.lib.kf_batch_incoming_frame_device(self.b, self._ptrs(dev_ptrs)))

    def synchronize(self) -> None:
        self._check(self.lib.kf_batch_synchronize(self.b))

    def kernels_per_frame(self) -> int:
        n = C.c_int(0)
        self._check(self.lib.kf_batch_kernels_per_frame(self.b, C.byref(n)))
        return n.value

    def autotune(self) -> tuple:
        t = (C.c_int * 4)()
        self._check(self.lib.kf_batch_autotune(self.b, t))
        return tuple(t)

    def set_tuning(self, tuning) -> None:
        self._check(self.lib.kf_batch_set_tuning(self.b, (C.c_int * 4)(*tuning)))

    def set_forms(self, persistent_integration: bool, persistent_icp: bool) -> None:
        """kf_batch_set_forms: spread integration / the ICP group pass over a fixed grid
        covering every scene's work (True) or one row of blocks per scene (False)."""
        self._check(self.lib.kf_batch_set_forms(self.b, int(persistent_integration), int(persistent_icp)))

