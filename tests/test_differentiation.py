"""The differentiation form: trilinear TSDF rendering and its hand-written adjoint.

Checked against central finite differences (pose and voxels), against the analytic
point-to-plane ICP Jacobian on a planar TSDF (where trilinear interpolation is exact),
through the torch.autograd.Function, and by a depth-rendering pose refinement that
recovers a perturbed pose.
"""
import numpy as np
import pytest

from kinect_fusion_slam_gb300 import diff

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

VD = 20.0
DIMS = (96, 96, 96)
START = (-48, -48, 10)
K = np.array([[131.25, 0.0, 80.5], [0.0, 131.25, 60.5], [0.0, 0.0, 1.0]])
H, W = 120, 160


def _centres():
    idx = [torch.arange(n, dtype=torch.float64, device="cuda") for n in DIMS]
    x = (idx[0] + START[0] + 0.5) * VD
    y = (idx[1] + START[1] + 0.5) * VD
    z = (idx[2] + START[2] + 0.5) * VD
    Z, Y, X = torch.meshgrid(z, y, x, indexing="ij")  # (dz, dy, dx): x fastest
    return X, Y, Z


def _tsdf(sdf, trunc=100.0):
    return torch.clamp(sdf / trunc, -1.0, 1.0).float().contiguous()


def scene_tsdf():
    """A sphere, a tilted floor and a back wall (union of their SDFs)."""
    X, Y, Z = _centres()
    sphere = torch.sqrt((X - 100) ** 2 + (Y + 50) ** 2 + (Z - 1200) ** 2) - 300
    n = torch.tensor([0.1, -1.0, -0.15], dtype=torch.float64)
    n = n / n.norm()
    floor = n[0] * X + n[1] * (Y - 400) + n[2] * (Z - 1200)
    wall = 1900 - Z
    return _tsdf(torch.minimum(torch.minimum(sphere, floor), wall))


def plane_tsdf(m, p0):
    X, Y, Z = _centres()
    return _tsdf(m[0] * (X - p0[0]) + m[1] * (Y - p0[1]) + m[2] * (Z - p0[2]))


def desc():
    return diff.make_desc(H, W, K, DIMS, START, VD, t_near=250.0, t_far=2100.0, step=0.5 * VD)


T0 = diff.se3_exp([0.02, -0.03, 0.01, 10.0, -5.0, 20.0])


def _loss(d, tsdf, T, gD, gN, mask):
    depth, normal = diff.render(d, tsdf, T)
    return float((depth.double() * gD * mask).sum() + (normal.double() * gN * mask[..., None]).sum())


def test_render_matches_the_analytic_sphere():
    X, Y, Z = _centres()
    tsdf = _tsdf(torch.sqrt(X ** 2 + Y ** 2 + (Z - 1000) ** 2) - 400)
    depth, normal = diff.render(desc(), tsdf, np.eye(4))
    u = torch.arange(W, device="cuda", dtype=torch.float64) + 1
    v = torch.arange(H, device="cuda", dtype=torch.float64) + 1
    dx = ((u - K[0, 2]) / K[0, 0])[None, :].expand(H, W)
    dy = ((v - K[1, 2]) / K[1, 1])[:, None].expand(H, W)
    a = dx ** 2 + dy ** 2 + 1
    disc = 1000.0 ** 2 - a * (1000.0 ** 2 - 400.0 ** 2)
    t_true = (1000.0 - torch.sqrt(torch.clamp(disc, min=0))) / a
    hit = (disc > 2e4 * a) & (depth > 0)
    assert hit.sum() > 3000
    err = (depth.double() - t_true)[hit].abs()
    # a truncated distance field interpolated between 20 mm voxels: sub-millimetre
    assert err.median() < 0.5 and err.max() < 3.0, (float(err.median()), float(err.max()))
    p = torch.stack([dx * t_true, dy * t_true, t_true - 1000], -1)
    n_true = p / p.norm(dim=-1, keepdim=True)
    cosang = (normal.double() * n_true).sum(-1)[hit]
    assert cosang.min() > np.cos(np.radians(3.0))


def _smooth_mask(d, tsdf, poses, margin=0.05):
    """Pixels that hit in every evaluation with the crossing point more than `margin`
    voxels from a cell face each time.  The trilinear gradient (the rendered normal) is
    discontinuous across cell faces, so a finite difference over a pixel whose crossing
    changes cell measures a jump, not the derivative."""
    Ki = np.linalg.inv(K)
    uv1 = np.stack(list(np.meshgrid(np.arange(W) + 1.0, np.arange(H) + 1.0)) + [np.ones((H, W))], -1) @ Ki.T
    uv1 = torch.from_numpy(uv1).cuda()
    start = torch.tensor(START, dtype=torch.float64, device="cuda")
    mask = torch.ones(H, W, device="cuda", dtype=torch.float64)
    cells = None
    for T in poses:
        depth, normal = diff.render(d, tsdf, T)
        R = torch.from_numpy(np.asarray(T)[:3, :3]).cuda()
        o = torch.from_numpy(np.asarray(T)[:3, 3]).cuda()
        x = o + depth.double()[..., None] * (uv1 @ R.T)
        gidx = x / VD - start - 0.5
        frac = gidx - torch.floor(gidx)
        near_face = ((frac < margin) | (frac > 1 - margin)).any(-1)
        c = torch.floor(gidx)
        same = torch.ones_like(mask, dtype=torch.bool) if cells is None else (c == cells).all(-1)
        cells = c if cells is None else cells
        mask *= ((depth > 0) & (normal.norm(dim=-1) > 0.5) & ~near_face & same).double()
    return mask


def _incidence_mask(d, tsdf, T, min_cos):
    """Pixels whose ray meets the surface at |cos(incidence)| >= min_cos: near grazing
    incidence the crossing point moves fast and nonlinearly with the pose."""
    Ki = np.linalg.inv(K)
    rays = np.stack(list(np.meshgrid(np.arange(W) + 1.0, np.arange(H) + 1.0)) + [np.ones((H, W))], -1) @ Ki.T
    rays = rays @ np.asarray(T)[:3, :3].T
    rays = torch.from_numpy(rays / np.linalg.norm(rays, axis=-1, keepdims=True)).cuda()
    _, normal = diff.render(d, tsdf, T)
    return ((normal.double() * rays).sum(-1).abs() >= min_cos).double()


def _pose_fd(d, tsdf, gD, gN, eps, min_cos=0.0):
    poses = [T0] + [diff.se3_exp(s * eps[k] * np.eye(6)[k]) @ T0 for k in range(6) for s in (1, -1)]
    mask = _smooth_mask(d, tsdf, poses) * _incidence_mask(d, tsdf, T0, min_cos)
    _, gp = diff.render_backward(d, tsdf, T0, (gD * mask).float(), (gN * mask[..., None]).float(), want_tsdf=False)
    fd = np.array([(_loss(d, tsdf, poses[1 + 2 * k], gD, gN, mask) - _loss(d, tsdf, poses[2 + 2 * k], gD, gN, mask))
                   / (2 * eps[k]) for k in range(6)])
    return gp.double().cpu().numpy(), fd, mask


def test_pose_gradient_of_depth_against_central_differences():
    d, tsdf = desc(), scene_tsdf()
    g = torch.Generator(device="cuda").manual_seed(3)
    gD = torch.randn(H, W, generator=g, device="cuda", dtype=torch.float64)
    gN = torch.zeros(H, W, 3, device="cuda", dtype=torch.float64)
    g6, fd, mask = _pose_fd(d, tsdf, gD, gN, np.array([1e-3, 1e-3, 1e-3, 0.5, 0.5, 0.5]))
    assert mask.sum() > 5000
    assert np.all(np.abs(g6 - fd) <= 0.02 * np.abs(fd) + 1e-3 * np.abs(fd).max()), (g6, fd)


def test_pose_gradient_of_normals_against_central_differences():
    d, tsdf = desc(), scene_tsdf()
    g = torch.Generator(device="cuda").manual_seed(4)
    gD = torch.zeros(H, W, device="cuda", dtype=torch.float64)
    gN = torch.randn(H, W, 3, generator=g, device="cuda", dtype=torch.float64)
    g6, fd, mask = _pose_fd(d, tsdf, gD, gN, np.array([2e-4, 2e-4, 2e-4, 0.1, 0.1, 0.1]), min_cos=0.35)
    assert mask.sum() > 3000
    assert np.all(np.abs(g6 - fd) <= 0.05 * np.abs(fd) + 0.01 * np.abs(fd).max()), (g6, fd)


def test_voxel_gradient_against_central_differences():
    d, tsdf = desc(), scene_tsdf()
    g = torch.Generator(device="cuda").manual_seed(5)
    gD = torch.randn(H, W, generator=g, device="cuda", dtype=torch.float64)
    gN = torch.randn(H, W, 3, generator=g, device="cuda", dtype=torch.float64)
    gt, _ = diff.render_backward(d, tsdf, T0, gD.float(), gN.float())
    flat = gt.view(-1)
    picks = torch.topk(flat.abs(), 2000).indices[::100].tolist()
    eps = 2e-3
    for idx in picks:
        tp, tm = tsdf.clone(), tsdf.clone()
        tp.view(-1)[idx] += eps
        tm.view(-1)[idx] -= eps
        mask = _smooth_mask(d, tsdf, [T0], margin=0.02) * _smooth_mask(d, tp, [T0], 0.02) * _smooth_mask(d, tm, [T0], 0.02)
        g_an, _ = diff.render_backward(d, tsdf, T0, (gD * mask).float(), (gN * mask[..., None]).float())
        fd = (_loss(d, tp, T0, gD, gN, mask) - _loss(d, tm, T0, gD, gN, mask)) / (2 * eps)
        an = float(g_an.view(-1)[idx])
        assert abs(an - fd) <= 0.03 * abs(fd) + 0.01 * float(flat.abs().max()), (idx, an, fd)


def test_depth_jacobian_is_the_icp_point_to_plane_jacobian():
    """For a plane, moving the camera by xi changes the rendered depth by
    -[x cross m, m] . xi / (m . r): the point-to-plane ICP row [x cross m, m]
    (sensor_pose_estimation.cu:72-78 up to its sign convention) over the ray's
    incidence on the plane."""
    m = np.array([0.2, -0.3, -1.0])
    m /= np.linalg.norm(m)
    p0 = np.array([0.0, 0.0, 1300.0])
    d, tsdf = desc(), plane_tsdf(m, p0)
    depth, _ = diff.render(d, tsdf, T0)
    dep = depth.cpu().numpy()
    Ki = np.linalg.inv(K)
    R, o = T0[:3, :3], T0[:3, 3]
    checked = 0
    for (v, u) in [(30, 40), (60, 80), (90, 120), (20, 140), (100, 30)]:
        D = float(dep[v, u])
        assert D > 0
        g1 = torch.zeros(H, W, device="cuda")
        g1[v, u] = 1.0
        _, gp = diff.render_backward(d, tsdf, T0, g1, None, want_tsdf=False)
        r = R @ (Ki @ np.array([u + 1.0, v + 1.0, 1.0]))
        x = o + D * r
        want = -np.concatenate([np.cross(x, m), m]) / float(m @ r)
        got = gp.double().cpu().numpy()
        assert np.allclose(got, want, rtol=2e-3, atol=2e-3 * np.abs(want).max()), (got, want)
        checked += 1
    assert checked == 5


def test_autograd_function_matches_the_adjoint():
    d, tsdf = desc(), scene_tsdf().requires_grad_(True)
    xi = torch.zeros(6, dtype=torch.float64, requires_grad=True)
    depth, normal = diff.trilinear_render(tsdf, xi, T0, d)
    g = torch.Generator(device="cuda").manual_seed(9)
    gD = torch.randn(H, W, generator=g, device="cuda")
    gN = torch.randn(H, W, 3, generator=g, device="cuda")
    ((depth * gD).sum() + (normal * gN).sum()).backward()
    gt, gp = diff.render_backward(d, tsdf.detach(), T0, gD, gN)
    assert torch.allclose(xi.grad.float(), gp.cpu(), rtol=1e-4, atol=1e-3)
    assert torch.allclose(tsdf.grad, gt, rtol=1e-4, atol=1e-4)


def test_depth_rendering_pose_refinement_recovers_the_pose():
    d, tsdf = desc(), scene_tsdf()
    T_true = T0
    measured, _ = diff.render(d, tsdf, T_true)
    start = diff.se3_exp([0.012, -0.008, 0.006, 15.0, -10.0, 12.0]) @ T_true
    T, rms = diff.refine_pose(d, tsdf, start, measured, iterations=15)
    dt = np.linalg.norm(T[:3, 3] - T_true[:3, 3])
    Rr = T[:3, :3].T @ T_true[:3, :3]
    ang = np.degrees(np.arccos(np.clip((np.trace(Rr) - 1) / 2, -1, 1)))
    assert rms[0] > 5.0 and rms[-1] < 0.05, rms
    assert dt < 0.1 and ang < 0.01, (dt, ang)
