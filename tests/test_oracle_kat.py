"""Known-answer tests of the CPU oracle: hand-built cases with analytic results."""
import numpy as np
import pytest

from oracle.pyoracle import GridSpec


def K_simple():
    return np.array([[500.0, 0, 320.5], [0, 500.0, 240.5], [0, 0, 1]], np.float32)


def test_opencv_restatements(oracle):
    K = K_simple()
    Ki = oracle.inv3(K)
    assert np.allclose(Ki @ K, np.eye(3), atol=1e-6)
    rng = np.random.default_rng(0)
    for _ in range(20):
        a = rng.normal(size=3)
        th = rng.uniform(0, np.pi)
        S = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]]) / np.linalg.norm(a)
        R = np.eye(3) + np.sin(th) * S + (1 - np.cos(th)) * S @ S
        T = np.eye(4, dtype=np.float32)
        T[:3, :3] = R
        T[:3, 3] = rng.uniform(-2000, 2000, 3)
        Ti = oracle.inv4(T)
        P = Ti.astype(np.float64) @ T
        assert np.allclose(P[:, :3], np.eye(4)[:, :3], atol=1e-6)
        assert np.allclose(P[:3, 3], 0, atol=2e-3)  # float LU on translations of ~2000 mm
        B = T.copy()
        assert np.allclose(oracle.matmul4(T, B), T.astype(np.float64) @ B, rtol=1e-6, atol=1e-3)
    # Cholesky solve of a well-conditioned SPD system, and the failure path
    M = rng.normal(size=(6, 6))
    A = (M @ M.T + 6 * np.eye(6)).astype(np.float32)
    b = rng.normal(size=6).astype(np.float32)
    ok, x = oracle.cholesky6(A, b)
    assert ok == 1 and np.allclose(A @ x, b, atol=1e-4)
    ok, x = oracle.cholesky6(np.zeros((6, 6), np.float32), b)
    assert ok == 0 and np.array_equal(x, b)  # b untouched on failure


def test_single_voxel_projection(oracle):
    """A fronto-parallel wall at 1000 mm seen from the identity pose: a voxel whose
    centre lies 40 mm in front of the wall on the optical axis gets 40/300."""
    H, W = 480, 640
    K = K_simple()
    Ki = oracle.inv3(K)
    g = GridSpec(dims=(4, 4, 4), start=(-2, -2, 94), voxel_size=10.0)  # z centres 945..975 mm
    depth = np.full((H, W), 1000.0, np.float32)
    T = np.eye(4, dtype=np.float32)
    t = np.full(g.nvox, np.nan, np.float32)
    w = np.full(g.nvox, np.nan, np.float32)
    oracle.integrate(g, depth, K, Ki, T, oracle.inv4(T), t, w, first=True)
    # voxel (2, 2, k): centre (5, 5, 945 + 10 k)
    for k in range(4):
        idx = (2 * 4 + 2) * 4 + k
        z = 945.0 + 10 * k
        assert w[idx] == 1.0
        # sdf along the pixel ray: D - |c - t| / |lambda|, lambda through the voxel's pixel
        assert abs(t[idx] - (1000.0 - z) / 300.0) < 2e-4


def test_behind_band_cut(oracle):
    """Voxels more than 30 mm behind the surface are not integrated (sdf_minimum)."""
    H, W = 48, 64
    K = np.array([[50.0, 0, 32.5], [0, 50.0, 24.5], [0, 0, 1]], np.float32)
    Ki = oracle.inv3(K)
    g = GridSpec(dims=(1, 1, 20), start=(0, 0, 90), voxel_size=10.0)  # centres z = 905 .. 1095
    depth = np.full((H, W), 1000.0, np.float32)
    T = np.eye(4, dtype=np.float32)
    T[0, 3] = 5.0
    T[1, 3] = 5.0  # camera on the column's axis
    t = np.full(g.nvox, np.nan, np.float32)
    w = np.full(g.nvox, np.nan, np.float32)
    oracle.integrate(g, depth, K, Ki, T, oracle.inv4(T), t, w, first=True)
    z = 905.0 + 10 * np.arange(20)
    expect = (1000 - z >= -30) & (1000 - z <= 300)
    assert np.array_equal(~np.isnan(w), expect)


def test_axis_ray_zero_crossing(oracle):
    """A plane sdf(z) = (1000 - z)/300 sampled on the grid: the ray through the image
    centre finds the surface at z = 1000 by linear interpolation along z."""
    H, W = 48, 64
    K = np.array([[50.0, 0, 32.5], [0, 50.0, 24.5], [0, 0, 1]], np.float32)
    Ki = oracle.inv3(K)
    g = GridSpec(dims=(40, 40, 60), start=(-20, -20, 70), voxel_size=10.0)
    zc = (np.arange(60) + 70) * 10.0 + 5.0
    sdf = np.clip((1000.0 - zc) / 300.0, -1, 1).astype(np.float32)
    t = np.broadcast_to(sdf, (40, 40, 60)).copy().ravel()
    depth = np.full((H, W), 1000.0, np.float32)
    T = np.eye(4, dtype=np.float32)
    pred, hit = oracle.raycast(g, depth, Ki, T, t)
    assert (hit >= 0).sum() > 0
    m = hit >= 0
    assert np.allclose(pred[2][m], 1000.0, atol=1e-3)
    # normals are the normalised central difference of the sdf, flipped towards the camera
    assert np.allclose(pred[5][m], -1.0, atol=1e-6)


def test_icp_single_pixel_system(oracle):
    """One correspondence: the 42 sums are exactly a*b and a a^T of that pixel."""
    H, W = 64, 64
    K = np.array([[50.0, 0, 32.5], [0, 50.0, 32.5], [0, 0, 1]], np.float32)
    cur6 = np.zeros((6, H, W), np.float32)
    pred6 = np.zeros((6, H, W), np.float32)
    mask = np.zeros((H, W), np.uint8)
    y, x = 10, 20
    v = np.array([(x + 1 - 32.5) / 50 * 1000, (y + 1 - 32.5) / 50 * 1000, 1000.0], np.float32)
    cur6[:3, y, x] = v
    cur6[3:, y, x] = [0, 0, -1]
    mask[y, x] = 1
    q = v + np.array([0, 0, 5.0], np.float32)
    m = np.array([0, 0, -1.0], np.float32)
    pred6[:3, y, x] = q
    pred6[3:, y, x] = m
    T = np.eye(4, dtype=np.float32)
    n, sums, pair = oracle.icp_associate(K, T, T, cur6, mask, pred6)
    assert n == 1 and pair[y, x] == y * W + x
    g = v
    a = np.array([g[2] * m[1] - g[1] * m[2], -g[2] * m[0] + g[0] * m[2], g[1] * m[0] - g[0] * m[1], *m], np.float32)
    b = np.float32(m @ (q - g))
    assert np.allclose(sums[:6], a * b)
    assert np.allclose(sums[6:].reshape(6, 6), np.outer(a, a))


def test_identity_icp_zero_increment(oracle):
    """Noise-free data registered against itself: every iteration's increment is ~0."""
    from kinect_fusion_slam_gb300 import scene

    cfg = scene.config("c0", noise=False, dropout=0.0)
    cam = scene.Camera().scaled(0.25)
    cfg = scene.SceneConfig(**{**cfg.__dict__, "camera": cam, "frames": 1})
    seq = scene.sequence(cfg)
    g = cfg.grid
    gs = GridSpec(tuple(g.dims), tuple(g.start), g.voxel_size)
    K = seq.K
    Ki = oracle.inv3(K)
    d = oracle.depth_ingest(seq.depth(0))
    t = np.full(gs.nvox, np.nan, np.float32)
    w = np.full(gs.nvox, np.nan, np.float32)
    T = np.eye(4, dtype=np.float32)
    oracle.integrate(gs, d, K, Ki, T, T, t, w, first=True)
    pred6, _ = oracle.raycast(gs, d, Ki, T, t)
    v5, mask = oracle.vertex_normal(d, Ki)
    cur6 = np.stack([v5[0], v5[1], d, v5[2], v5[3], v5[4]])
    Te, log = oracle.estimate_pose(K, T, cur6, mask, pred6, iters=3)
    assert log["ncorr"][0] > 1000
    # the ray-cast prediction is not the measured surface exactly (per-axis interpolation),
    # so the estimate moves a little, but stays within a millimetre and a few millidegrees
    assert np.abs(Te[:3, 3]).max() < 2.0
    assert np.abs(Te[:3, :3] - np.eye(3)).max() < 2e-3


def test_acos_threshold_equivalence(oracle):
    """The ICP normal gate acos(c)*(180/pi) <= 30 is 'c >= c30' over all floats in
    [0.5, 1] (acos is monotone); checked exhaustively with the oracle's libm."""
    lo = np.float32(0.5).view(np.int32)
    hi = np.float32(1.0).view(np.int32)
    cs = np.arange(lo, hi + 1, dtype=np.int32).view(np.float32)
    f = np.frompyfunc(lambda c: oracle.lib.kfo_icp_angle_deg(float(c)), 1, 1)
    sample = cs[:: 997]
    ang = np.array(f(sample), dtype=np.float32)
    ok = (ang <= 30.0) & (ang >= 0.0)
    # monotone: once accepted, every larger cosine is accepted
    first = np.argmax(ok)
    assert ok[first:].all() and not ok[:first].any()
