"""ctypes front end for the CPU oracle and the CPU-compiled reference kernels.

TEST INFRASTRUCTURE: imported only by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``.  The product never imports this module.

``Oracle`` wraps ``libkf_oracle.so`` (the restatement) and ``Reference`` wraps
``_ref/libkf_ref.so`` (the reference's own kernel bodies, when it could be built).
Both expose the same methods on numpy arrays, in the reference's conventions
(millimetres, 1-based pixels, z-fastest volume ``idx = x*DY*DZ + y*DZ + z``).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import build as _build

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


class Grid(C.Structure):
    _fields_ = [
        ("dims", C.c_int * 3),
        ("start", C.c_int * 3),
        ("voxel_size", C.c_float),
        ("truncated_distance", C.c_float),
        ("sdf_minimum", C.c_float),
        ("sdf_maximum", C.c_float),
    ]


@dataclass(frozen=True)
class GridSpec:
    dims: tuple = (360, 360, 300)
    start: tuple = (-200, -200, -120)
    voxel_size: float = 10.0
    truncated_distance: float = 300.0
    sdf_minimum: float = -30.0
    sdf_maximum: float = 300.0

    def c(self) -> Grid:
        g = Grid()
        g.dims[:] = list(self.dims)
        g.start[:] = list(self.start)
        g.voxel_size = self.voxel_size
        g.truncated_distance = self.truncated_distance
        g.sdf_minimum = self.sdf_minimum
        g.sdf_maximum = self.sdf_maximum
        return g

    @property
    def nvox(self) -> int:
        return int(np.prod(self.dims))


def _nullable(arr):
    return None if arr is None else arr.ctypes.data_as(C.c_void_p)


class _Common:
    prefix = "kfo"

    def __init__(self, lib: C.CDLL):
        self.lib = lib
        p = self.prefix
        self._fn(f"{p}_integrate", None, [C.POINTER(Grid), C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p, _f32p,
                                           _f32p, _f32p, C.c_int])
        self._fn(f"{p}_raycast", None, [C.POINTER(Grid), C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p, _f32p, _i32p])
        self._fn(f"{p}_vertex_normal", None, [C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _f32p, _u8p])
        self._fn(f"{p}_icp_associate", C.c_int, [C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p, _u8p, _f32p,
                                                 C.c_void_p, _f32p])
        self._fn(f"{p}_bilateral", None, [C.c_int, C.c_int, _f32p, _f32p, C.c_int, C.c_float, _f32p])

    def _fn(self, name, res, args):
        f = getattr(self.lib, name)
        f.restype = res
        f.argtypes = args
        return f

    # -- kernels --------------------------------------------------------------
    def integrate(self, grid: GridSpec, depth, K, Kinv, T, Tinv, tsdf, weight, first: bool):
        H, W = depth.shape
        getattr(self.lib, f"{self.prefix}_integrate")(C.byref(grid.c()), H, W, _c32(depth), _c32(K), _c32(Kinv),
                                                      _c32(T), _c32(Tinv), tsdf, weight, int(first))

    def raycast(self, grid: GridSpec, depth, Kinv, T, tsdf):
        H, W = depth.shape
        out6 = np.zeros((6, H, W), np.float32)
        hit = np.full((H, W), -1, np.int32)
        getattr(self.lib, f"{self.prefix}_raycast")(C.byref(grid.c()), H, W, _c32(depth), _c32(Kinv), _c32(T),
                                                    _c32(tsdf), out6, hit)
        return out6, hit

    def vertex_normal(self, depth, Kinv):
        H, W = depth.shape
        out = np.zeros((5, H, W), np.float32)
        mask = np.zeros((H, W), np.uint8)
        getattr(self.lib, f"{self.prefix}_vertex_normal")(H, W, _c32(depth), _c32(Kinv), out[0], out[1], out[2],
                                                          out[3], out[4], mask)
        return out, mask

    def icp_associate(self, K, F, T, cur6, mask, pred6, want_pair=True):
        _, H, W = cur6.shape
        sums = np.zeros(42, np.float32)
        pair = np.full((H, W), -1, np.int32) if want_pair else None
        n = getattr(self.lib, f"{self.prefix}_icp_associate")(H, W, _c32(K), _c32(F), _c32(T), _c32(cur6),
                                                              np.ascontiguousarray(mask, np.uint8), _c32(pred6),
                                                              _nullable(pair), sums)
        return n, sums, pair

    def bilateral(self, depth, spatial, radius: int, sigma_r: float):
        H, W = depth.shape
        out = np.zeros((H, W), np.float32)
        getattr(self.lib, f"{self.prefix}_bilateral")(H, W, _c32(depth), _c32(spatial), radius, sigma_r, out)
        return out


def _c32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


class Oracle(_Common):
    prefix = "kfo"

    def __init__(self, path=None):
        super().__init__(C.CDLL(str(path or _build.build_oracle())))
        L = self.lib
        self._fn("kfo_inv3", None, [_f32p, _f32p])
        self._fn("kfo_inv4", C.c_int, [_f32p, _f32p])
        self._fn("kfo_matmul4", None, [_f32p, _f32p, _f32p])
        self._fn("kfo_cholesky6", C.c_int, [_f32p, _f32p])
        self._fn("kfo_icp_angle_deg", C.c_float, [C.c_float])
        self._fn("kfo_raycast_flip", C.c_int, [C.c_float])
        self._fn("kfo_depth_ingest", None, [_u16p, C.c_int, C.c_float, C.c_float, _f32p])
        self._fn("kfo_estimate_pose", None, [C.c_int, C.c_int, _f32p, _f32p, _f32p, _u8p, _f32p, C.c_int,
                                             C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p])
        self._fn("kfo_create", C.c_void_p, [C.c_int, C.c_int, C.c_float, C.c_float, C.POINTER(Grid), _f32p, C.c_int])
        self._fn("kfo_destroy", None, [C.c_void_p])
        self._fn("kfo_initial", None, [C.c_void_p, _u16p])
        self._fn("kfo_incoming", None, [C.c_void_p, _u16p])
        self._fn("kfo_set_bilateral", None, [C.c_void_p, C.c_int, C.c_int, C.c_float, C.c_float])
        self._fn("kfo_incoming_filtered", None, [C.c_void_p, _u16p, _f32p])
        self._fn("kfo_get_pose", None, [C.c_void_p, _f32p])
        self._fn("kfo_set_pose", None, [C.c_void_p, _f32p])
        self._fn("kfo_get_prediction", None, [C.c_void_p, C.c_void_p, C.c_void_p])
        self._fn("kfo_get_volume", None, [C.c_void_p, C.c_void_p, C.c_void_p])
        self._fn("kfo_get_depth", None, [C.c_void_p, _f32p])
        self._fn("kfo_get_vertex_map", None, [C.c_void_p, C.c_void_p, C.c_void_p])
        self._fn("kfo_num_threads", C.c_int, [])
        self._fn("kfo_set_pyramid", None, [C.c_void_p, C.c_int, np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"),
                                           C.c_float])
        self._fn("kfo_pyramid_depth", None, [C.c_int, C.c_int, _f32p, C.c_float, _f32p])
        self._fn("kfo_level_intrinsics", None, [_f32p, C.c_int, _f32p])
        self._fn("kfo_icp_terms", None, [C.c_int, C.c_int, _f32p, _f32p, _f32p, _f32p, _u8p, _f32p, _f32p])
        _f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        self._fn("kfo64_create", C.c_void_p, [C.c_int, C.c_int, C.c_double, C.c_double, C.POINTER(Grid), _f64p,
                                               C.c_int])
        self._fn("kfo64_destroy", None, [C.c_void_p])
        self._fn("kfo64_initial", None, [C.c_void_p, _u16p])
        self._fn("kfo64_incoming", None, [C.c_void_p, _u16p])
        self._fn("kfo64_get_pose", None, [C.c_void_p, _f64p])
        self._fn("kfo64_set_pose", None, [C.c_void_p, _f64p])
        self._fn("kfo64_integrate_frame", None, [C.c_void_p, _u16p, C.c_int])
        self._fn("kfo64_raycast_frame", None, [C.c_void_p])
        self._fn("kfo64_get_prediction", None, [C.c_void_p, _f64p])
        self._fn("kfo64_get_volume", None, [C.c_void_p, C.c_void_p, C.c_void_p])
        self.L = L

    def inv3(self, K):
        out = np.zeros(9, np.float32)
        self.lib.kfo_inv3(_c32(K).ravel(), out)
        return out.reshape(3, 3)

    def inv4(self, T):
        out = np.zeros(16, np.float32)
        self.lib.kfo_inv4(_c32(T).ravel(), out)
        return out.reshape(4, 4)

    def matmul4(self, A, B):
        out = np.zeros(16, np.float32)
        self.lib.kfo_matmul4(_c32(A).ravel(), _c32(B).ravel(), out)
        return out.reshape(4, 4)

    def cholesky6(self, A, b):
        A = _c32(A).ravel().copy()
        b = _c32(b).ravel().copy()
        ok = self.lib.kfo_cholesky6(A, b)
        return ok, b

    def depth_ingest(self, raw, min_depth=300.0, max_depth=2000.0):
        raw = np.ascontiguousarray(raw, np.uint16)
        out = np.zeros(raw.shape, np.float32)
        self.lib.kfo_depth_ingest(raw.ravel(), raw.size, min_depth, max_depth, out.ravel())
        return out

    def estimate_pose(self, K, T, cur6, mask, pred6, iters=10):
        _, H, W = cur6.shape
        T = _c32(T).copy()
        sums = np.zeros((iters, 42), np.float32)
        poses = np.zeros((iters, 16), np.float32)
        ncorr = np.zeros(iters, np.int32)
        ok = np.zeros(iters, np.int32)
        self.lib.kfo_estimate_pose(H, W, _c32(K), T, _c32(cur6), np.ascontiguousarray(mask, np.uint8), _c32(pred6),
                                   iters, _nullable(sums), _nullable(poses), _nullable(ncorr), _nullable(ok))
        return T, {"sums": sums, "poses": poses.reshape(iters, 4, 4), "ncorr": ncorr, "chol_ok": ok}

    def pyramid_depth(self, depth, band=90.0):
        depth = _c32(depth)
        H, W = depth.shape
        out = np.zeros((H // 2, W // 2), np.float32)
        self.lib.kfo_pyramid_depth(H, W, depth.ravel(), band, out.ravel())
        return out

    def level_intrinsics(self, K, level):
        out = np.zeros(9, np.float32)
        self.lib.kfo_level_intrinsics(_c32(K).ravel(), int(level), out)
        return out.reshape(3, 3)

    def icp_terms(self, K, F, T, cur6, mask, pred6):
        """(H*W, 42) per-pixel ICP products: a*b (6) then a a^T (36); zero off correspondences."""
        _, H, W = cur6.shape
        out = np.zeros((H * W, 42), np.float32)
        self.lib.kfo_icp_terms(H, W, _c32(K), _c32(F), _c32(T), _c32(cur6), np.ascontiguousarray(mask, np.uint8),
                               _c32(pred6), out)
        return out

    def pipeline(self, H, W, grid: GridSpec, K, min_depth=300.0, max_depth=2000.0, icp_iters=10):
        return OraclePipeline(self, H, W, grid, K, min_depth, max_depth, icp_iters)

    def pipeline64(self, H, W, grid: GridSpec, K, min_depth=300.0, max_depth=2000.0, icp_iters=10):
        """The FP64 oracle's frame loop (kf_oracle64.cpp)."""
        return Oracle64Pipeline(self, H, W, grid, K, min_depth, max_depth, icp_iters)


class Oracle64Pipeline:
    """The frame loop with every quantity in double (the precision form's yardstick)."""

    def __init__(self, o: Oracle, H, W, grid: GridSpec, K, min_depth, max_depth, icp_iters):
        self.o, self.H, self.W, self.grid = o, H, W, grid
        self._g = grid.c()
        K64 = np.ascontiguousarray(np.asarray(K, np.float32).astype(np.float64).ravel())
        self.h = o.lib.kfo64_create(H, W, min_depth, max_depth, C.byref(self._g), K64, icp_iters)

    def close(self):
        if self.h:
            self.o.lib.kfo64_destroy(self.h)
            self.h = None

    __del__ = close

    def initial(self, raw):
        self.o.lib.kfo64_initial(self.h, np.ascontiguousarray(raw, np.uint16).ravel())

    def incoming(self, raw):
        self.o.lib.kfo64_incoming(self.h, np.ascontiguousarray(raw, np.uint16).ravel())

    @property
    def pose(self):
        T = np.zeros(16, np.float64)
        self.o.lib.kfo64_get_pose(self.h, T)
        return T.reshape(4, 4)

    @pose.setter
    def pose(self, T):
        self.o.lib.kfo64_set_pose(self.h, np.ascontiguousarray(T, np.float64).ravel())

    def integrate_frame(self, raw, first: bool):
        self.o.lib.kfo64_integrate_frame(self.h, np.ascontiguousarray(raw, np.uint16).ravel(), int(first))

    def raycast_frame(self):
        self.o.lib.kfo64_raycast_frame(self.h)

    def prediction(self):
        out6 = np.zeros((6, self.H, self.W), np.float64)
        self.o.lib.kfo64_get_prediction(self.h, out6)
        return out6

    def volume(self):
        t = np.zeros(self.grid.nvox, np.float32)
        w = np.zeros(self.grid.nvox, np.float32)
        self.o.lib.kfo64_get_volume(self.h, _nullable(t), _nullable(w))
        return t, w


class OraclePipeline:
    """KinfuPipeline's frame loop (kinfu_pipeline.cpp:91-193) on the CPU oracle."""

    def __init__(self, o: Oracle, H, W, grid: GridSpec, K, min_depth, max_depth, icp_iters):
        self.o, self.H, self.W, self.grid = o, H, W, grid
        self._g = grid.c()
        self.h = o.lib.kfo_create(H, W, min_depth, max_depth, C.byref(self._g), _c32(K).ravel(), icp_iters)

    def close(self):
        if self.h:
            self.o.lib.kfo_destroy(self.h)
            self.h = None

    __del__ = close

    def initial(self, raw):
        self.o.lib.kfo_initial(self.h, np.ascontiguousarray(raw, np.uint16).ravel())

    def incoming(self, raw, filtered=None):
        """IncomingFrameProcessing; with the bilateral stage on, `filtered` (H x W float)
        replaces the stage's own output."""
        raw = np.ascontiguousarray(raw, np.uint16).ravel()
        if filtered is None:
            self.o.lib.kfo_incoming(self.h, raw)
        else:
            self.o.lib.kfo_incoming_filtered(self.h, raw, _c32(filtered).ravel())

    def set_bilateral(self, enable=True, radius=3, sigma_d=4.5, sigma_r=30.0):
        """The bilateral stage at the reference's commented-out call site."""
        self.o.lib.kfo_set_bilateral(self.h, int(enable), int(radius), float(sigma_d), float(sigma_r))

    def set_pyramid(self, levels, iterations, band=90.0):
        """ICP pyramid: iterations per level, finest first."""
        it = np.zeros(3, np.int32)
        it[:len(iterations)] = iterations
        self.o.lib.kfo_set_pyramid(self.h, int(levels), it, float(band))

    @property
    def pose(self):
        T = np.zeros(16, np.float32)
        self.o.lib.kfo_get_pose(self.h, T)
        return T.reshape(4, 4)

    @pose.setter
    def pose(self, T):
        self.o.lib.kfo_set_pose(self.h, _c32(T).ravel())

    def prediction(self):
        out6 = np.zeros((6, self.H, self.W), np.float32)
        hit = np.zeros((self.H, self.W), np.int32)
        self.o.lib.kfo_get_prediction(self.h, _nullable(out6), _nullable(hit))
        return out6, hit

    def volume(self):
        t = np.zeros(self.grid.nvox, np.float32)
        w = np.zeros(self.grid.nvox, np.float32)
        self.o.lib.kfo_get_volume(self.h, _nullable(t), _nullable(w))
        return t, w

    def depth(self):
        d = np.zeros((self.H, self.W), np.float32)
        self.o.lib.kfo_get_depth(self.h, d)
        return d

    def vertex_map(self):
        cur6 = np.zeros((6, self.H, self.W), np.float32)
        mask = np.zeros((self.H, self.W), np.uint8)
        self.o.lib.kfo_get_vertex_map(self.h, _nullable(cur6), _nullable(mask))
        return cur6, mask


class Reference(_Common):
    """The reference's kernel bodies compiled for the CPU (None-returning factory
    ``Reference.load()`` when they could not be built)."""

    prefix = "kfr"

    def __init__(self, path):
        super().__init__(C.CDLL(str(path)))
        self._fn("kfr_estimate_pose", None, [C.c_int, C.c_int, _f32p, _f32p, _f32p, _u8p, _f32p, C.c_int,
                                             C.c_void_p, C.c_void_p])
        self._fn("kfr_create", C.c_void_p, [C.c_int, C.c_int, C.c_float, C.c_float, C.POINTER(Grid), _f32p])
        self._fn("kfr_destroy", None, [C.c_void_p])
        self._fn("kfr_initial", None, [C.c_void_p, _u16p])
        self._fn("kfr_incoming", None, [C.c_void_p, _u16p, C.c_int])
        self._fn("kfr_get_pose", None, [C.c_void_p, _f32p])
        self._fn("kfr_get_prediction", None, [C.c_void_p, C.c_void_p, C.c_void_p])
        self._fn("kfr_get_volume", None, [C.c_void_p, C.c_void_p, C.c_void_p])

    @classmethod
    def load(cls):
        try:
            path = _build.build_ref()
        except Exception:  # no compiler / broken splice: the caller decides what to skip
            return None
        return cls(path) if path is not None else None

    def estimate_pose(self, K, T, cur6, mask, pred6, iters=10):
        _, H, W = cur6.shape
        T = _c32(T).copy()
        sums = np.zeros((iters, 42), np.float32)
        poses = np.zeros((iters, 16), np.float32)
        self.lib.kfr_estimate_pose(H, W, _c32(K), T, _c32(cur6), np.ascontiguousarray(mask, np.uint8), _c32(pred6),
                                   iters, _nullable(sums), _nullable(poses))
        return T, {"sums": sums, "poses": poses.reshape(iters, 4, 4)}

    def pipeline(self, H, W, grid: GridSpec, K, min_depth=300.0, max_depth=2000.0, icp_iters=10):
        return ReferencePipeline(self, H, W, grid, K, min_depth, max_depth, icp_iters)


class ReferencePipeline:
    def __init__(self, r: Reference, H, W, grid: GridSpec, K, min_depth, max_depth, icp_iters):
        self.r, self.H, self.W, self.grid, self.icp_iters = r, H, W, grid, icp_iters
        self._g = grid.c()
        self.h = r.lib.kfr_create(H, W, min_depth, max_depth, C.byref(self._g), _c32(K).ravel())

    def close(self):
        if self.h:
            self.r.lib.kfr_destroy(self.h)
            self.h = None

    __del__ = close

    def initial(self, raw):
        self.r.lib.kfr_initial(self.h, np.ascontiguousarray(raw, np.uint16).ravel())

    def incoming(self, raw):
        self.r.lib.kfr_incoming(self.h, np.ascontiguousarray(raw, np.uint16).ravel(), self.icp_iters)

    @property
    def pose(self):
        T = np.zeros(16, np.float32)
        self.r.lib.kfr_get_pose(self.h, T)
        return T.reshape(4, 4)

    def prediction(self):
        out6 = np.zeros((6, self.H, self.W), np.float32)
        hit = np.zeros((self.H, self.W), np.int32)
        self.r.lib.kfr_get_prediction(self.h, _nullable(out6), _nullable(hit))
        return out6, hit

    def volume(self):
        t = np.zeros(self.grid.nvox, np.float32)
        w = np.zeros(self.grid.nvox, np.float32)
        self.r.lib.kfr_get_volume(self.h, _nullable(t), _nullable(w))
        return t, w


def reference_K():
    """The reference's intrinsics, kinfu_pipeline.cpp:14-24 (1-based principal point)."""
    return np.array([[524.639, 0.0, 316.625], [0.0, 523.503, 256.2318], [0.0, 0.0, 1.0]], np.float32)
