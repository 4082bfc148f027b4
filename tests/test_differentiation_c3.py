"""The differentiation form on its configured workload (c3): the seeded analytic room
fused by the library's own integration into a 256^3 TSDF at 10 mm (64 frames at their
poses), 64 camera poses each perturbed by a seeded 2-5 cm / 1-3 degree step, rendered
640x480 depth compared with the unperturbed rendered target under a Huber loss
(delta = 10 mm).

* pose gradients of the loss (the hand-written adjoint) against central differences
  with step 1e-4 (1e-4 rad; 1e-4 m = 0.1 mm);
* voxel gradients against central differences with step 1e-4 (TSDF units);
* the depth Jacobian against the analytic point-to-plane ICP row -[x cross m, m]/(m.r)
  (sensor_pose_estimation.cu:72-78) on the room's flat faces;
* a 50-step Huber Gauss-Newton refinement from the 64 starts, beside the reference's
  ICP from the same starts.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from kinect_fusion_slam_gb300 import diff  # noqa: E402

DELTA = 10.0       # Huber threshold, mm
H_ROT = 1e-4       # rad
H_TRANS = 0.1      # mm (1e-4 m)


@pytest.fixture(scope="module")
def room():
    w = diff.RoomWorkload("c3")
    w.targets = [diff.render(w.desc, w.tsdf, T)[0].double() for T in w.poses]
    yield w
    w.close()


def _bracket(w, depth):
    """The index of the march's sample before each pixel's crossing."""
    return torch.floor((depth.double() - w.desc.t_near) / w.desc.step)


def _stable(w, depth, margin=0.05, bracket=None):
    """Pixels whose crossing lies away from the march's sample points (and, given a
    reference, between the same two samples as there): the rendered depth -- the linear
    crossing between two samples -- is a smooth function of the pose and the voxels only
    while the bracket stays, and a ray whose first crossing moves to another surface
    (an occlusion edge) jumps."""
    b = _bracket(w, depth)
    f = (depth.double() - w.desc.t_near) / w.desc.step - b
    ok = (depth > 0) & (f > margin) & (f < 1 - margin)
    return ok if bracket is None else ok & (b == bracket)


def _loss(w, T, target, mask):
    depth, _ = diff.render(w.desc, w.tsdf, T)
    rho, _ = diff.huber(depth.double() - target, DELTA)
    return float((rho * mask).sum())


@pytest.mark.parametrize("k", [0, 21, 42, 63])
def test_pose_gradient_against_central_differences(room, k):
    w = room
    T, target = w.starts[k], w.targets[k]
    eps = np.array([H_ROT] * 3 + [H_TRANS] * 3)
    poses = [T] + [diff.se3_exp(s * eps[q] * np.eye(6)[q]) @ T for q in range(6) for s in (1, -1)]
    mask = (target > 0)
    b0 = _bracket(w, diff.render(w.desc, w.tsdf, T)[0])
    for P in poses:
        mask &= _stable(w, diff.render(w.desc, w.tsdf, P)[0], bracket=b0)
    mask = mask.double()
    assert mask.sum() > 50_000
    depth, _ = diff.render(w.desc, w.tsdf, T)
    _, psi = diff.huber(depth.double() - target, DELTA)
    _, g6 = diff.render_backward(w.desc, w.tsdf, T, (psi * mask).float(), None, want_tsdf=False)
    g6 = g6.double().cpu().numpy()
    fd = np.array([(_loss(w, poses[1 + 2 * q], target, mask) - _loss(w, poses[2 + 2 * q], target, mask))
                   / (2 * eps[q]) for q in range(6)])
    print(f"pose {k}: adjoint {g6.round(2)} central differences {fd.round(2)}")
    assert np.all(np.abs(g6 - fd) <= 0.02 * np.abs(fd) + 2e-3 * np.abs(fd).max()), (g6, fd)


def test_voxel_gradient_against_central_differences(room):
    w = room
    T, target = w.starts[10], w.targets[10]
    depth, _ = diff.render(w.desc, w.tsdf, T)
    b0 = _bracket(w, depth)
    mask = ((target > 0) & _stable(w, depth, 0.02)).double()
    _, psi = diff.huber(depth.double() - target, DELTA)
    gt, _ = diff.render_backward(w.desc, w.tsdf, T, (psi * mask).float(), None)
    flat = gt.view(-1)
    picks = torch.topk(flat.abs(), 3000).indices[::100].tolist()
    eps = 1e-4
    worst = 0.0
    for idx in picks:
        tp, tm = w.tsdf.clone(), w.tsdf.clone()
        tp.view(-1)[idx] += eps
        tm.view(-1)[idx] -= eps
        m = mask * _stable(w, diff.render(w.desc, tp, T)[0], 0.02, b0).double() * \
            _stable(w, diff.render(w.desc, tm, T)[0], 0.02, b0).double()
        g_an, _ = diff.render_backward(w.desc, w.tsdf, T, (psi * m).float(), None)
        lp = float((diff.huber(diff.render(w.desc, tp, T)[0].double() - target, DELTA)[0] * m).sum())
        lm = float((diff.huber(diff.render(w.desc, tm, T)[0].double() - target, DELTA)[0] * m).sum())
        fd = (lp - lm) / (2 * eps)
        an = float(g_an.view(-1)[idx])
        worst = max(worst, abs(an - fd) / max(abs(fd), 1e-9))
        assert abs(an - fd) <= 0.03 * abs(fd) + 0.01 * float(flat.abs().max()), (idx, an, fd)
    print(f"voxel gradients: {len(picks)} voxels, worst relative difference {worst:.3e}")


def test_depth_jacobian_is_the_point_to_plane_row_on_flat_faces(room):
    """On locally flat parts of the fused surfaces (the rendered normal within 3 degrees
    over a 9x9 window) the depth Jacobian of a pixel is close to the point-to-plane ICP
    row -[x cross m, m]/(m.r), m the surface normal at the crossing.  The two agree
    exactly where the TSDF is affine (tests/test_differentiation.py, planar TSDF); the
    fused volume of noisy depth is not affine within a cell, and the rendered crossing
    interpolates between two samples whose gradients differ from the crossing's, so the
    check here is on the distribution of the relative difference over the pixels."""
    w = room
    T = w.poses[0]
    depth, normal = diff.render(w.desc, w.tsdf, T)
    n = normal.double().cpu().numpy()
    dep = depth.cpu().numpy()
    Hh, Ww = dep.shape
    Ki = np.linalg.inv(np.asarray(w.K, np.float64))
    R, o = T[:3, :3], T[:3, 3]
    cos3 = np.cos(np.radians(3.0))
    checked, rel = 0, []
    for v in range(40, Hh - 40, 11):
        for u in range(40, Ww - 40, 14):
            if dep[v, u] <= 0 or not np.all(dep[v - 4:v + 5, u - 4:u + 5] > 0):
                continue
            m = n[v, u] / np.linalg.norm(n[v, u])
            if (n[v - 4:v + 5, u - 4:u + 5] @ m).min() < cos3:
                continue
            g1 = torch.zeros_like(depth)
            g1[v, u] = 1.0
            _, gp = diff.render_backward(w.desc, w.tsdf, T, g1, None, want_tsdf=False)
            r = R @ (Ki @ np.array([u + 1.0, v + 1.0, 1.0]))
            x = o + float(dep[v, u]) * r
            want = -np.concatenate([np.cross(x, m), m]) / float(m @ r)
            got = gp.double().cpu().numpy()
            rel.append(float(np.linalg.norm(got - want) / np.linalg.norm(want)))
            checked += 1
    rel = np.array(rel)
    print(f"point-to-plane rows at {checked} pixels: relative difference median {np.median(rel):.4f}, "
          f"90th percentile {np.percentile(rel, 90):.4f}, max {rel.max():.4f}")
    assert checked >= 20, checked
    assert np.median(rel) <= 0.03 and np.percentile(rel, 90) <= 0.10


def test_refinement_beside_icp_from_the_64_starts(room):
    """50 Huber Gauss-Newton steps of the depth rendering (kf_render_depth_normal_equations
    _huber) from each of the 64 perturbed starts, and the reference's 10-iteration ICP from
    the same starts: the refinement recovers the pose (within 2 mm and 0.2 degrees) from
    nearly every start."""
    w = room
    ref, icp = [], []
    for k, (T0, Tt) in enumerate(zip(w.starts, w.poses)):
        T, _ = diff.refine_pose(w.desc, w.tsdf, T0, w.targets[k].float(), iterations=50, max_residual=0.0,
                                huber_delta=DELTA)
        ref.append(diff.pose_error(T, Tt))
        icp.append(diff.pose_error(diff.icp_align(w.handle, T0, w.targets[k].cpu().numpy()), Tt))
    ref, icp = np.array(ref), np.array(icp)
    ok = lambda e: float(np.mean((e[:, 0] <= 2.0) & (e[:, 1] <= 0.2)))  # noqa: E731
    print(f"refinement: success {ok(ref):.3f}, median {np.median(ref[:, 0]):.3f} mm {np.median(ref[:, 1]):.4f} deg;"
          f" ICP: success {ok(icp):.3f}, median {np.median(icp[:, 0]):.3f} mm {np.median(icp[:, 1]):.4f} deg")
    assert ok(ref) >= 0.9 and np.median(ref[:, 0]) < 0.5
