"""The differentiation form over the C ABI: trilinear TSDF rendering with its adjoint as
a torch.autograd.Function, and a depth-rendering pose refinement that stands beside ICP.

The TSDF is a CUDA float32 tensor of shape (dz, dy, dx) -- this library's x-fastest
layout, NaN for unobserved voxels.  Poses are 4x4 camera-to-world (mm); a pose
parameter xi = (omega, tau) perturbs a base pose on the left, T(xi) = exp(xi^) T0,
with omega and tau in world coordinates (the frame of the reference's ICP increment,
sensor_pose_estimation.cu:406-428).  Gradients with respect to xi are exact at xi = 0
(the adjoint differentiates the left perturbation of the pose it renders at).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


RenderDesc = _lib.RenderDesc


def make_desc(height, width, K, dims, grid_start, voxel_size, t_near, t_far, step=None) -> RenderDesc:
    """K: 3x3 intrinsics in the reference's convention (1-based principal point)."""
    K = np.asarray(K, np.float64)
    d = RenderDesc()
    d.height, d.width = int(height), int(width)
    d.fx, d.fy, d.cx, d.cy = float(K[0, 0]), float(K[1, 1]), float(K[0, 2]), float(K[1, 2])
    d.dims[:] = [int(v) for v in dims]
    d.grid_start[:] = [int(v) for v in grid_start]
    d.voxel_size = float(voxel_size)
    d.t_near, d.t_far = float(t_near), float(t_far)
    d.step = float(step if step is not None else 0.5 * voxel_size)
    return d


def se3_exp(xi) -> np.ndarray:
    """exp(xi^) for xi = (omega, tau), as a 4x4 float64 matrix (Rodrigues)."""
    xi = np.asarray(xi, np.float64).ravel()
    w, v = xi[:3], xi[3:]
    th = float(np.linalg.norm(w))
    Wx = np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])
    if th < 1e-12:
        R = np.eye(3) + Wx
        V = np.eye(3) + 0.5 * Wx
    else:
        a, b, c = np.sin(th) / th, (1 - np.cos(th)) / th ** 2, (th - np.sin(th)) / th ** 3
        R = np.eye(3) + a * Wx + b * Wx @ Wx
        V = np.eye(3) + b * Wx + c * Wx @ Wx
    T = np.eye(4)
    T[:3, :3] = R
    T[:3, 3] = V @ v
    return T


def _f32_pose(T) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(T, np.float64), np.float32).ravel()


def _stream():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _dptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def render(desc: RenderDesc, tsdf, T):
    """(depth (H, W), normal (H, W, 3)) rendered at pose T."""
    import torch

    _check_volume(desc, tsdf)
    depth = torch.empty((desc.height, desc.width), dtype=torch.float32, device=tsdf.device)
    normal = torch.empty((desc.height, desc.width, 3), dtype=torch.float32, device=tsdf.device)
    lib = _lib.load()
    st = lib.kf_render_trilinear(C.byref(desc), _dptr(tsdf), _f32_pose(T), _dptr(depth), _dptr(normal), _stream())
    if st != _lib.KF_OK:
        raise _lib.KinfuError(st, "kf_render_trilinear")
    return depth, normal


def render_backward(desc: RenderDesc, tsdf, T, grad_depth=None, grad_normal=None, want_tsdf=True):
    """(dL/d tsdf or None, dL/d xi (6,)) for upstream gradients of depth and normal."""
    import torch

    _check_volume(desc, tsdf)
    gt = torch.zeros_like(tsdf) if want_tsdf else None
    gp = torch.zeros(6, dtype=torch.float32, device=tsdf.device)
    gd = grad_depth.contiguous().float() if grad_depth is not None else None
    gn = grad_normal.contiguous().float() if grad_normal is not None else None
    lib = _lib.load()
    st = lib.kf_render_trilinear_backward(C.byref(desc), _dptr(tsdf), _f32_pose(T), _dptr(gd), _dptr(gn), _dptr(gt),
                                          _dptr(gp), _stream())
    if st != _lib.KF_OK:
        raise _lib.KinfuError(st, "kf_render_trilinear_backward")
    return gt, gp


def _check_volume(desc, tsdf):
    import torch

    if not (isinstance(tsdf, torch.Tensor) and tsdf.is_cuda and tsdf.dtype == torch.float32 and tsdf.is_contiguous()):
        raise ValueError("tsdf must be a contiguous CUDA float32 tensor")
    if tuple(tsdf.shape) != (desc.dims[2], desc.dims[1], desc.dims[0]):
        raise ValueError(f"tsdf shape {tuple(tsdf.shape)} does not match dims (dz, dy, dx)")


def _autograd_function():
    import torch

    class TrilinearRender(torch.autograd.Function):
        """depth, normal = TrilinearRender.apply(tsdf, xi, T0, desc): the trilinear render
        at exp(xi^) T0, differentiable in tsdf and xi (xi's gradient is exact at 0)."""

        @staticmethod
        def forward(ctx, tsdf, xi, T0, desc):
            T = se3_exp(xi.detach().cpu().numpy()) @ np.asarray(T0, np.float64)
            depth, normal = render(desc, tsdf, T)
            ctx.save_for_backward(tsdf)
            ctx.T, ctx.desc = T, desc
            ctx.xi_device, ctx.xi_dtype = xi.device, xi.dtype
            return depth, normal

        @staticmethod
        def backward(ctx, grad_depth, grad_normal):
            (tsdf,) = ctx.saved_tensors
            gt, gp = render_backward(ctx.desc, tsdf, ctx.T, grad_depth, grad_normal,
                                     want_tsdf=ctx.needs_input_grad[0])
            return gt, gp.to(device=ctx.xi_device, dtype=ctx.xi_dtype), None, None

    return TrilinearRender


_TR = None


def trilinear_render(tsdf, xi, T0, desc):
    """Differentiable render (see TrilinearRender)."""
    global _TR
    if _TR is None:
        _TR = _autograd_function()
    return _TR.apply(tsdf, xi, T0, desc)


def depth_normal_equations(desc: RenderDesc, tsdf, T, measured_depth, max_residual: float = 0.0,
                           huber_delta: float = 0.0) -> np.ndarray:
    """The 29 Gauss-Newton sums of the depth residual (kf_render_depth_normal_equations;
    with huber_delta > 0 the Huber-weighted sums of kf_render_depth_normal_equations_huber)."""
    _check_volume(desc, tsdf)
    sums = np.zeros(29, np.float64)
    meas = measured_depth.contiguous().float()  # held until the synchronous call returns
    lib = _lib.load()
    st = lib.kf_render_depth_normal_equations_huber(C.byref(desc), _dptr(tsdf), _f32_pose(T), _dptr(meas),
                                                    float(max_residual), float(huber_delta),
                                                    sums.ctypes.data_as(C.POINTER(C.c_double)), _stream())
    if st != _lib.KF_OK:
        raise _lib.KinfuError(st, "kf_render_depth_normal_equations_huber")
    return sums


def refine_pose(desc: RenderDesc, tsdf, T0, measured_depth, iterations: int = 10, max_residual: float = 50.0,
                huber_delta: float = 0.0):
    """Gauss-Newton alignment of the rendered depth to a measured depth map: each step
    solves (J^T W J) dxi = -J^T W r in double over the pixels with |r| <= max_residual mm
    (W = 1, or the Huber weights min(1, huber_delta / |r|): iteratively reweighted least
    squares on the Huber loss) and applies T <- exp(dxi^) T.  Returns the pose and the
    per-step RMS residual (mm; with Huber weights the root of the mean 2 rho(r))."""
    T = np.asarray(T0, np.float64).copy()
    rms = []
    for _ in range(iterations):
        s = depth_normal_equations(desc, tsdf, T, measured_depth, max_residual, huber_delta)
        n = s[27]
        if n < 6:
            break
        A = np.zeros((6, 6))
        q = 0
        for a in range(6):
            for b in range(a, 6):
                A[a, b] = A[b, a] = s[q]
                q += 1
        rms.append(float(np.sqrt(s[28] / n)))
        try:
            dxi = -np.linalg.solve(A, s[21:27])
        except np.linalg.LinAlgError:
            break
        T = se3_exp(dxi) @ T
    return T, rms


# ---- the differentiation workload's pieces: a fused volume, perturbed starts, the Huber
# loss, and the reference's ICP from a given start ----------------------------------------
def fuse(h, depths, poses) -> None:
    """Integrate depth frames (uint16 mm) into handle h's volume at the given poses with the
    library's projective TSDF update (Projective_TSDF, projective_tsdf.cu:5-140); the first
    frame with first-frame semantics."""
    for k, (d, T) in enumerate(zip(depths, poses)):
        h.set_pose(np.asarray(T, np.float32))
        h.set_depth_u16(d)
        h.projective_tsdf(first=(k == 0))


def volume_tensor(h):
    """Handle h's FP32 TSDF as a CUDA float32 tensor (dz, dy, dx) -- the layout the renderer
    takes (x fastest, NaN unobserved)."""
    import torch

    t, _ = h.volume(weight=False)
    dx, dy, dz = h.dims
    return torch.from_numpy(np.ascontiguousarray(t.reshape(dx, dy, dz).transpose(2, 1, 0))).cuda()


def perturbed_starts(poses, seed: int, trans_mm=(20.0, 50.0), rot_deg=(1.0, 3.0)) -> list:
    """A seeded perturbation of each pose, exp(xi^) T with xi = (angle a, distance t):
    a rotation of 1-3 degrees about a random axis and a translation of 20-50 mm in a
    random direction (world frame), uniform in the ranges."""
    from .scene import gaussian, uniform

    out = []
    for k, T in enumerate(poses):
        g = gaussian(seed, 20, np.arange(6 * k, 6 * k + 6, dtype=np.uint64))
        u = uniform(seed, 21, np.arange(2 * k, 2 * k + 2, dtype=np.uint64))
        axis = g[:3] / np.linalg.norm(g[:3])
        tdir = g[3:] / np.linalg.norm(g[3:])
        ang = np.radians(rot_deg[0] + (rot_deg[1] - rot_deg[0]) * u[0])
        dist = trans_mm[0] + (trans_mm[1] - trans_mm[0]) * u[1]
        out.append(se3_exp(np.concatenate([axis * ang, tdir * dist])) @ np.asarray(T, np.float64))
    return out


def pose_error(T, T_ref):
    """(translation error mm, rotation error degrees) of T against T_ref."""
    T, T_ref = np.asarray(T, np.float64), np.asarray(T_ref, np.float64)
    R = T[:3, :3] @ T_ref[:3, :3].T
    s = 0.5 * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    return float(np.linalg.norm(T[:3, 3] - T_ref[:3, 3])), float(np.degrees(np.arctan2(np.linalg.norm(s),
                                                                                      (np.trace(R) - 1) / 2)))


def huber(r, delta: float):
    """(rho(r), psi(r)) elementwise: rho = r^2 / 2 for |r| <= delta, delta (|r| - delta / 2)
    beyond; psi = d rho / d r = clamp(r, -delta, delta)."""
    import torch

    a = r.abs()
    rho = torch.where(a <= delta, 0.5 * r * r, delta * (a - 0.5 * delta))
    return rho, r.clamp(-delta, delta)


def icp_align(h, T_start, depth) -> np.ndarray:
    """The reference's ICP (Estimate_Sensor_Pose, sensor_pose_estimation.cu:247-436: 10
    point-to-plane iterations) on handle h, from T_start, of a depth map (H x W float mm)
    against the surface ray cast from h's volume at T_start (the previous frame's pose, as
    in the frame loop).  Returns the estimated pose."""
    h.set_pose(np.asarray(T_start, np.float32))
    h.set_depth_f32(np.asarray(depth, np.float32))
    h.ray_casting()
    h.calculate_vertices_and_normals()
    return h.estimate_sensor_pose()


class RoomWorkload:
    """The differentiation workload: the seeded analytic room's depth frames fused by this
    library's projective TSDF integration into an FP32 volume (the c3 grid: 256^3 at
    10 mm), the renderer's description of it, the frames' poses and a seeded perturbed
    start per pose (2-5 cm, 1-3 degrees).  `handle` keeps the fused volume for the
    library's ICP; `tsdf` is the same volume as a CUDA tensor for the renderer."""

    def __init__(self, name: str = "c3", frames: int | None = None, t_near: float = 300.0, t_far: float = 2600.0):
        from . import Handle, make_config
        from . import scene as _scene

        seq = _scene.sequence(name, frames=frames)
        n = seq.cfg.frames
        depths = _scene.render_sequences([seq.cfg], n)[0]
        g, cam = seq.cfg.grid, seq.cfg.camera
        self.seq, self.poses, self.K = seq, [np.asarray(T, np.float64) for T in seq.poses[:n]], seq.K
        self.handle = Handle(make_config(height=cam.height, width=cam.width, dims=g.dims, grid_start=g.start,
                                         voxel_size=g.voxel_size))
        self.handle.set_intrinsics(seq.K[0, 0], seq.K[1, 1], seq.K[0, 2], seq.K[1, 2])
        fuse(self.handle, depths, self.poses)
        self.tsdf = volume_tensor(self.handle)
        self.desc = make_desc(cam.height, cam.width, seq.K, g.dims, g.start, g.voxel_size, t_near, t_far,
                              step=0.5 * g.voxel_size)
        self.starts = perturbed_starts(self.poses, seed=seq.cfg.seed)

    def close(self):
        self.handle.close()
