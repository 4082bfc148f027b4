"""GPU parity: the CUDA library (through the C ABI) against the CPU oracle.

Each stage gets identical inputs on both sides.  Gates (from the reference's
tolerances): integer results bit for bit -- integration weight counts and the set of
integrated voxels, ray-cast hit voxel indices, ICP correspondence pairings; floats
within TSDF |d| <= 1e-6, points <= 1e-5 m (1e-2 mm), normals <= 1e-5, pose
<= 1e-5 rad / 1e-5 m.
"""
import dataclasses

import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from conftest import grid_spec

pytestmark = pytest.mark.gpu

TSDF_TOL = 1e-6
POINT_TOL_MM = 1e-2
NORMAL_TOL = 1e-5
ROT_TOL = 1e-5
TRANS_TOL_MM = 1e-2


def make_handle(seq, **kw):
    g, cam = seq.cfg.grid, seq.cfg.camera
    h = kf.Handle(kf.make_config(height=cam.height, width=cam.width, dims=g.dims, grid_start=g.start,
                                 voxel_size=g.voxel_size, **kw))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    return h


def assert_volume_parity(tg, wg, to, wo):
    assert np.array_equal(np.isnan(wg), np.isnan(wo)), "integrated voxel sets differ"
    assert np.array_equal(np.isnan(tg), np.isnan(to))
    m = ~np.isnan(wo)
    assert np.array_equal(wg[m], wo[m]), "weight counts differ"
    d = np.abs(tg[m] - to[m])
    assert d.size == 0 or d.max() <= TSDF_TOL, d.max()


def test_depth_and_vertex_map(oracle, small_seq):
    seq, depths = small_seq
    h = make_handle(seq)
    Ki = oracle.inv3(seq.K)
    for d in depths:
        h.set_depth_u16(d)
        dg = h.depth()
        do = oracle.depth_ingest(d)
        assert np.array_equal(dg, do)
        out_g, mask_g = h.calculate_vertices_and_normals()
        out_o, mask_o = oracle.vertex_normal(do, Ki)
        assert np.array_equal(mask_g, mask_o)
        assert np.abs(out_g[:2] - out_o[:2]).max() <= POINT_TOL_MM
        assert np.abs(out_g[2:] - out_o[2:]).max() <= NORMAL_TOL
        # same operations in the same order without FMA: expected to be bit-identical
        assert np.array_equal(out_g.view(np.uint32), out_o.view(np.uint32))


@pytest.mark.parametrize("frame_pair", [(0, 1), (1, 3)])
def test_integration(oracle, small_seq, frame_pair):
    seq, depths = small_seq
    gs = grid_spec(seq.cfg.grid)
    h = make_handle(seq)
    K = seq.K
    Ki = oracle.inv3(K)
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    for n, k in enumerate(frame_pair):
        T = seq.poses[k].astype(np.float32)
        depth = oracle.depth_ingest(depths[k])
        h.set_pose(T)
        h.set_depth_f32(depth)
        h.projective_tsdf(first=(n == 0))
        oracle.integrate(gs, depth, K, Ki, T, oracle.inv4(T), to, wo, first=(n == 0))
        tg, wg = h.volume()
        assert_volume_parity(tg, wg, to, wo)
    assert np.count_nonzero(~np.isnan(wo)) > 1000


def _rot(yaw, pitch, roll):
    cy, sy, cp, sp, cr, sr = np.cos(yaw), np.sin(yaw), np.cos(pitch), np.sin(pitch), np.cos(roll), np.sin(roll)
    Rz = np.array([[cr, -sr, 0], [sr, cr, 0], [0, 0, 1]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rx = np.array([[1, 0, 0], [0, cp, -sp], [0, sp, cp]])
    return Ry @ Rx @ Rz


@pytest.mark.parametrize("offset_vox", [0, 2500, 16000])
def test_integration_cull_exact(oracle, small_seq, offset_vox):
    """Integration skips voxel boxes and column segments that provably hold no updated
    voxel (behind the camera, outside the image, or beyond the truncation band of every
    depth their pixels can read).  Hard cases for those proofs, bit for bit against the
    oracle: oblique camera poses inside the grid, depths from 0.1 to 6 m with holes,
    negative and isolated near samples, and the whole scene moved 50 m or 320 m from the
    origin (larger rounding against the translation; at 320 m the marks' depth band has
    no far bound of its own and the grid's far side bounds it)."""
    seq, _ = small_seq
    g = seq.cfg.grid
    cam = seq.cfg.camera
    off = float(offset_vox) * g.voxel_size
    start = tuple(int(v) + offset_vox for v in g.start)
    h = kf.Handle(kf.make_config(height=cam.height, width=cam.width, dims=g.dims, grid_start=start,
                                 voxel_size=g.voxel_size))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    gs = dataclasses.replace(grid_spec(g), start=start)
    Ki = oracle.inv3(K)
    rng = np.random.default_rng(5 + offset_vox)
    H, W = cam.height, cam.width
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    poses = [(0.3, 0.2, 0.0, (200.0, -150.0, -300.0)), (-0.5, -0.25, 0.3, (-400.0, 300.0, 100.0)),
             (1.2, 0.1, -0.2, (0.0, 0.0, 500.0))]
    for n, (yaw, pitch, roll, t) in enumerate(poses):
        T = np.eye(4)
        T[:3, :3] = _rot(yaw, pitch, roll)
        T[:3, 3] = np.asarray(t) + off
        T = T.astype(np.float32)
        # smooth surface plus steps, holes and outliers
        yy, xx = np.mgrid[0:H, 0:W]
        depth = 1500.0 + 900.0 * np.sin(xx / 17.0) * np.cos(yy / 11.0) + 2000.0 * (xx > W // 2)
        depth = depth.astype(np.float32)
        depth[rng.random((H, W)) < 0.2] = 0.0
        depth[rng.random((H, W)) < 0.01] = 100.0
        depth[rng.random((H, W)) < 0.01] = 6000.0
        depth[rng.random((H, W)) < 0.005] *= -1.0
        depth[: H // 4, : W // 4] = 0.0
        h.set_pose(T)
        h.set_depth_f32(depth)
        h.projective_tsdf(first=(n == 0))
        oracle.integrate(gs, depth, K, Ki, T, oracle.inv4(T), to, wo, first=(n == 0))
        tg, wg = h.volume()
        assert_volume_parity(tg, wg, to, wo)
    assert np.count_nonzero(~np.isnan(wo)) > 1000


def test_integration_cull_exact_wide_angle(oracle, small_seq):
    """A wide-angle camera (focal length 30 px on 160 x 120: rays up to 3.5 times their
    depth long at the corners) with many depths of 50-150 mm: the voxels updated closer
    than the marking's first slab lie up to ~350 mm from the camera centre, beyond the
    default near radius, and must still be listed.  Bit for bit against the oracle."""
    seq, _ = small_seq
    g = seq.cfg.grid
    cam = seq.cfg.camera
    H, W = cam.height, cam.width
    h = kf.Handle(kf.make_config(height=H, width=W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size))
    K = np.array([[30.0, 0.0, W / 2 + 0.5], [0.0, 30.0, H / 2 + 0.5], [0.0, 0.0, 1.0]], np.float32)
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    gs = grid_spec(g)
    Ki = oracle.inv3(K)
    rng = np.random.default_rng(17)
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    poses = [(0.3, 0.2, 0.0, (200.0, -150.0, -300.0)), (-0.5, -0.25, 0.3, (-400.0, 300.0, 100.0)),
             (1.2, 0.1, -0.2, (0.0, 0.0, 500.0))]
    for n, (yaw, pitch, roll, t) in enumerate(poses):
        T = np.eye(4)
        T[:3, :3] = _rot(yaw, pitch, roll)
        T[:3, 3] = t
        T = T.astype(np.float32)
        yy, xx = np.mgrid[0:H, 0:W]
        depth = (400.0 + 300.0 * np.sin(xx / 9.0) * np.cos(yy / 7.0)).astype(np.float32)
        near = rng.random((H, W)) < 0.1
        depth[near] = rng.uniform(50.0, 150.0, int(near.sum())).astype(np.float32)
        depth[rng.random((H, W)) < 0.1] = 0.0
        h.set_pose(T)
        h.set_depth_f32(depth)
        h.projective_tsdf(first=(n == 0))
        oracle.integrate(gs, depth, K, Ki, T, oracle.inv4(T), to, wo, first=(n == 0))
        tg, wg = h.volume()
        assert_volume_parity(tg, wg, to, wo)
    assert np.count_nonzero(~np.isnan(wo)) > 1000


def test_integration_huge_depths(oracle, small_seq):
    """Depths of 1e7 mm, 1e30 mm and +inf beside the sequence's own (float input, no
    range filter): the marks' slabs end at the grid's far side, so the marking pass stays
    as short as for ordinary depths, and the volume is bit for bit the oracle's."""
    seq, depths = small_seq
    gs = grid_spec(seq.cfg.grid)
    h = make_handle(seq)
    K = seq.K
    Ki = oracle.inv3(K)
    rng = np.random.default_rng(23)
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    for n, k in enumerate([0, 1, 2]):
        T = seq.poses[k].astype(np.float32)
        depth = oracle.depth_ingest(depths[k]).copy()
        for value, frac in [(1e7, 0.02), (1e30, 0.02), (np.inf, 0.02)]:
            depth[rng.random(depth.shape) < frac] = value
        h.set_pose(T)
        h.set_depth_f32(depth)
        h.projective_tsdf(first=(n == 0))
        oracle.integrate(gs, depth, K, Ki, T, oracle.inv4(T), to, wo, first=(n == 0))
        tg, wg = h.volume()
        assert_volume_parity(tg, wg, to, wo)
    assert np.count_nonzero(~np.isnan(wo)) > 1000


def test_raycast(oracle, small_seq):
    seq, depths = small_seq
    gs = grid_spec(seq.cfg.grid)
    h = make_handle(seq)
    K = seq.K
    Ki = oracle.inv3(K)
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    for n, k in enumerate([0, 1, 2]):
        T = seq.poses[k].astype(np.float32)
        oracle.integrate(gs, oracle.depth_ingest(depths[k]), K, Ki, T, oracle.inv4(T), to, wo, first=(n == 0))
    h.set_volume(to, wo)
    for k in [2, 3]:
        T = seq.poses[k].astype(np.float32)
        depth = oracle.depth_ingest(depths[k])
        h.set_pose(T)
        h.set_depth_f32(depth)
        hit_g = h.ray_casting()
        pred_g = h.predicted()
        pred_o, hit_o = oracle.raycast(gs, depth, Ki, T, to)
        assert np.array_equal(hit_g, hit_o), f"{int((hit_g != hit_o).sum())} hit indices differ"
        assert (hit_o >= 0).sum() > 500
        m = hit_o >= 0
        assert np.abs(pred_g[:3][:, m] - pred_o[:3][:, m]).max() <= POINT_TOL_MM
        nm = m & ~np.isnan(pred_o[3])
        assert np.abs(pred_g[3:][:, nm] - pred_o[3:][:, nm]).max() <= NORMAL_TOL
        assert np.array_equal(np.isnan(pred_g), np.isnan(pred_o))
        assert np.all(pred_g[:, ~m] == 0)


def test_integration_raycast_c1(oracle):
    """The bench's size: 640x480 into 360x360x300 @ 10 mm, three frames at ground-truth
    poses plus one at a perturbed pose; every integrated voxel, weight and hit index bit
    for bit."""
    from kinect_fusion_slam_gb300 import scene

    seq = scene.sequence("c1", frames=4)
    depths = seq.depths(4)
    gs = grid_spec(seq.cfg.grid)
    h = make_handle(seq)
    K = seq.K
    Ki = oracle.inv3(K)
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    rng = np.random.default_rng(5)
    for n, k in enumerate(range(4)):
        T = seq.poses[k].astype(np.float32)
        if k == 3:
            T[:3, 3] += rng.normal(0, 20, 3).astype(np.float32)
        d = oracle.depth_ingest(depths[k])
        h.set_pose(T)
        h.set_depth_f32(d)
        h.projective_tsdf(first=(n == 0))
        oracle.integrate(gs, d, K, Ki, T, oracle.inv4(T), to, wo, first=(n == 0))
        hit_g = h.ray_casting()
        pred_o, hit_o = oracle.raycast(gs, d, Ki, T, to)
        assert np.array_equal(hit_g, hit_o), f"frame {k}: {int((hit_g != hit_o).sum())} hits differ"
    tg, wg = h.volume()
    assert_volume_parity(tg, wg, to, wo)
    assert int((~np.isnan(wo)).sum()) > 100000 and int((hit_o >= 0).sum()) > 100000


def test_flip_threshold(oracle, small_seq):
    """The ray-cast normal flip uses a float threshold the device derives from its own
    double acos; it must equal the threshold of the oracle's libm acos."""
    seq, _ = small_seq
    h = make_handle(seq)
    c = np.float32(h.flip_threshold())
    assert oracle.lib.kfo_raycast_flip(float(np.nextafter(c, np.float32(-1)))) == 1
    assert oracle.lib.kfo_raycast_flip(float(c)) == 0


def _icp_inputs(oracle, seq, depths, k_prev=0, k_cur=1):
    gs = grid_spec(seq.cfg.grid)
    K = seq.K
    Ki = oracle.inv3(K)
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    Tp = seq.poses[k_prev].astype(np.float32)
    dp = oracle.depth_ingest(depths[k_prev])
    oracle.integrate(gs, dp, K, Ki, Tp, oracle.inv4(Tp), to, wo, first=True)
    pred6, _ = oracle.raycast(gs, dp, Ki, Tp, to)
    dc = oracle.depth_ingest(depths[k_cur])
    v5, mask = oracle.vertex_normal(dc, Ki)
    cur6 = np.stack([v5[0], v5[1], dc, v5[2], v5[3], v5[4]])
    return Tp, dc, cur6, mask, pred6


def test_icp_association(oracle, small_seq):
    seq, depths = small_seq
    Tp, dc, cur6, mask, pred6 = _icp_inputs(oracle, seq, depths)
    h = make_handle(seq)
    h.set_depth_f32(dc)
    h.calculate_vertices_and_normals()
    h.set_predicted(pred6)
    rng = np.random.default_rng(3)
    for trial in range(3):
        T = Tp.copy()
        if trial:
            T[:3, 3] += rng.normal(0, 3, 3).astype(np.float32)
        F = oracle.matmul4(oracle.inv4(Tp), T)
        n_g, sums_g, pair_g = h.icp_associate(F, T)
        n_o, sums42, pair_o = oracle.icp_associate(seq.K, F, T, cur6, mask, pred6)
        assert n_o > 200
        assert n_g == n_o
        assert np.array_equal(pair_g, pair_o), f"{int((pair_g != pair_o).sum())} pairings differ"
        A = sums42[6:].reshape(6, 6)
        ref27 = np.concatenate([sums42[:6], A[np.triu_indices(6)]])
        # the reference's summation order: bit-identical sums
        assert np.array_equal(sums_g.view(np.uint32), ref27.view(np.uint32))


def test_icp_association_tree_order(oracle, small_seq):
    """The one-pass tree reduction: same pairings, sums equal to rounding."""
    seq, depths = small_seq
    Tp, dc, cur6, mask, pred6 = _icp_inputs(oracle, seq, depths)
    h = make_handle(seq, icp_reduction=kf.KF_REDUCE_TREE)
    h.set_depth_f32(dc)
    h.calculate_vertices_and_normals()
    h.set_predicted(pred6)
    F = oracle.matmul4(oracle.inv4(Tp), Tp)
    n_g, sums_g, pair_g = h.icp_associate(F, Tp)
    n_o, sums42, pair_o = oracle.icp_associate(seq.K, F, Tp, cur6, mask, pred6)
    assert n_g == n_o and np.array_equal(pair_g, pair_o)
    A = sums42[6:].reshape(6, 6)
    ref27 = np.concatenate([sums42[:6], A[np.triu_indices(6)]])
    assert np.abs(sums_g - ref27).max() <= 1e-4 * np.abs(ref27).max()


def test_estimate_pose(oracle, small_seq):
    seq, depths = small_seq
    Tp, dc, cur6, mask, pred6 = _icp_inputs(oracle, seq, depths)
    h = make_handle(seq)
    h.set_pose(Tp)
    h.set_depth_f32(dc)
    h.calculate_vertices_and_normals()
    h.set_predicted(pred6)
    Tg = h.estimate_sensor_pose()
    To, log = oracle.estimate_pose(seq.K, Tp, cur6, mask, pred6, iters=10)
    nc, ok, Ts = h.icp_stats(10, poses=True)
    assert np.array_equal(nc, log["ncorr"]) and np.array_equal(ok, log["chol_ok"])
    # reference summation order + the same solve: every iteration's pose bit for bit
    assert np.array_equal(Ts.view(np.uint32), log["poses"].view(np.uint32))
    assert np.array_equal(Tg.view(np.uint32), To.view(np.uint32))


def test_estimate_pose_tree_order(oracle, small_seq):
    seq, depths = small_seq
    Tp, dc, cur6, mask, pred6 = _icp_inputs(oracle, seq, depths)
    h = make_handle(seq, icp_reduction=kf.KF_REDUCE_TREE)
    h.set_pose(Tp)
    h.set_depth_f32(dc)
    h.calculate_vertices_and_normals()
    h.set_predicted(pred6)
    h.estimate_sensor_pose()
    To, log = oracle.estimate_pose(seq.K, Tp, cur6, mask, pred6, iters=10)
    nc, ok, Ts = h.icp_stats(10, poses=True)
    assert nc[0] == log["ncorr"][0]
    # the first iteration sees identical inputs: its pose agrees to rounding
    assert np.abs(Ts[0] - log["poses"][0]).max() <= 1e-5 * max(1.0, np.abs(To).max())


def test_icp_fail_identity(small_seq):
    """KF_ICP_FAIL_IDENTITY: a failed factorisation leaves the pose unchanged."""
    seq, depths = small_seq
    h = make_handle(seq, icp_fail_mode=kf.KF_ICP_FAIL_IDENTITY)
    h.initial_processing(depths[0])
    T = seq.poses[1].astype(np.float32)
    T[:3, 3] += 5000.0  # far outside the scene: no correspondences, A = 0
    h.set_pose(T)
    h.incoming_frame(depths[1])
    nc, ok = h.icp_stats(10)
    assert np.all(nc == 0) and np.all(ok == 0)
    assert np.array_equal(h.pose(), T)


def test_bilateral(oracle, small_seq):
    seq, depths = small_seq
    h = make_handle(seq)
    d = oracle.depth_ingest(depths[1])
    h.set_depth_f32(d)
    h.bilateral_filtering()
    out_g = h.depth()
    r, sd = 3, 4.5
    yy, xx = np.mgrid[-r:r + 1, -r:r + 1].astype(np.float32)
    spatial = np.exp((-(xx * xx + yy * yy) / np.float32(2 * sd * sd)).astype(np.float64)).astype(np.float32)
    out_o = oracle.bilateral(d, spatial, r, 30.0)
    assert np.abs(out_g - out_o).max() <= 1e-2


def run_synced(oracle, seq, depths, h, exact=True):
    """Runs the GPU frame loop and, at every frame, the oracle's stages on the GPU's own
    state at the start of that frame: the ICP pose must agree within tolerance, and
    integration and ray casting at the GPU's pose must agree bit for bit.  Returns the
    worst pose deviations."""
    gs = grid_spec(seq.cfg.grid)
    K = seq.K
    Ki = oracle.inv3(K)
    T = np.eye(4, dtype=np.float32)
    d = oracle.depth_ingest(depths[0])
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    h.initial_processing(depths[0])
    oracle.integrate(gs, d, K, Ki, T, oracle.inv4(T), to, wo, first=True)
    tg, wg = h.volume()
    assert_volume_parity(tg, wg, to, wo)
    worst = [0.0, 0.0]
    for k in range(1, len(depths)):
        pred_prev = h.predicted()
        T_prev = h.pose()
        tg_prev, wg_prev = tg, wg
        h.incoming_frame(depths[k])
        Tg = h.pose()
        d = oracle.depth_ingest(depths[k])
        v5, mask = oracle.vertex_normal(d, Ki)
        cur6 = np.stack([v5[0], v5[1], d, v5[2], v5[3], v5[4]])
        To, log = oracle.estimate_pose(K, T_prev, cur6, mask, pred_prev, iters=10)
        nc, _ = h.icp_stats(10)
        assert nc[0] == log["ncorr"][0], f"frame {k}: first-iteration correspondences differ"
        if exact:
            assert np.array_equal(Tg.view(np.uint32), To.view(np.uint32)), f"frame {k}: pose bits differ"
        worst[0] = max(worst[0], float(np.abs(Tg[:3, :3] - To[:3, :3]).max()))
        worst[1] = max(worst[1], float(np.abs(Tg[:3, 3] - To[:3, 3]).max()))
        # integration and ray cast at the GPU's pose, from the GPU's volume
        to, wo = tg_prev.copy(), wg_prev.copy()
        oracle.integrate(gs, d, K, Ki, Tg, oracle.inv4(Tg), to, wo, first=False)
        tg, wg = h.volume()
        assert_volume_parity(tg, wg, to, wo)
        pred_o, hit_o = oracle.raycast(gs, d, Ki, Tg, tg)
        hit_g = h.ray_casting()
        assert np.array_equal(hit_g, hit_o), f"frame {k}: {int((hit_g != hit_o).sum())} hits differ"
        m = hit_o >= 0
        assert np.abs(h.predicted()[:3][:, m] - pred_o[:3][:, m]).max() <= POINT_TOL_MM
    return worst


def test_pipeline_small(oracle, small_seq):
    seq, depths = small_seq
    worst = run_synced(oracle, seq, depths, make_handle(seq))
    print(f"small: worst per-frame pose deviation rot {worst[0]:.2e}, trans {worst[1]:.2e} mm")
    assert worst[0] <= ROT_TOL and worst[1] <= TRANS_TOL_MM


def test_pipeline_c0(oracle, c0_seq):
    """Config c0 (640x480, 180x180x150 @ 20 mm), 20 frames, stage-synced, reference
    summation order: poses bit for bit at every frame."""
    seq, depths = c0_seq
    worst = run_synced(oracle, seq, depths, make_handle(seq))
    print(f"c0: worst per-frame pose deviation rot {worst[0]:.2e}, trans {worst[1]:.2e} mm")
    assert worst == [0.0, 0.0]


def test_pipeline_free_running_c0(oracle, c0_seq):
    """GPU and oracle each run the whole c0 sequence on their own: the same trajectory,
    volume and prediction bit for bit."""
    seq, depths = c0_seq
    gs = grid_spec(seq.cfg.grid)
    h = make_handle(seq)
    o = oracle.pipeline(480, 640, gs, seq.K)
    h.initial_processing(depths[0])
    o.initial(depths[0])
    for k in range(1, len(depths)):
        h.incoming_frame(depths[k])
        o.incoming(depths[k])
        assert np.array_equal(h.pose().view(np.uint32), o.pose.view(np.uint32)), f"frame {k}"
    tg, wg = h.volume()
    to, wo = o.volume()
    assert_volume_parity(tg, wg, to, wo)
    pred_o, hit_o = o.prediction()
    assert np.array_equal(h.ray_casting(), hit_o)


def test_pipeline_free_running_c2(oracle):
    """The largest grid of the workloads, c2 (512x512x430 @ 7 mm: 113 M voxels, linear
    indices past 2^26), plain form: four frames free-running on the GPU and in the float
    oracle give the same poses, voxels, weights and hit indices bit for bit."""
    from kinect_fusion_slam_gb300 import scene

    seq = scene.sequence("c2", frames=4)
    depths = seq.depths(4)
    gs = grid_spec(seq.cfg.grid)
    assert gs.nvox > 1 << 26
    h = make_handle(seq)
    o = oracle.pipeline(480, 640, gs, seq.K)
    h.initial_processing(depths[0])
    o.initial(depths[0])
    for k in range(1, len(depths)):
        h.incoming_frame(depths[k])
        o.incoming(depths[k])
        assert np.array_equal(h.pose().view(np.uint32), o.pose.view(np.uint32)), f"frame {k}"
    tg, wg = h.volume()
    to, wo = o.volume()
    assert_volume_parity(tg, wg, to, wo)
    assert int((~np.isnan(wo)).sum()) > 1_000_000
    _, hit_o = o.prediction()
    hit_g = h.ray_casting()
    assert np.array_equal(hit_g, hit_o) and int((hit_o >= 0).sum()) > 100_000
    h.close()


def test_graph_and_eager_agree(small_seq):
    seq, depths = small_seq
    poses = []
    for graphs in (1, 0):
        h = make_handle(seq, use_graphs=graphs)
        h.initial_processing(depths[0])
        for k in range(1, len(depths)):
            h.incoming_frame(depths[k])
        poses.append(h.pose())
        h.close()
    assert np.array_equal(poses[0], poses[1])


def test_process_frame_and_zero_based_intrinsics(small_seq):
    """kf_process_frame(is_first) is kf_initial_processing / kf_incoming_frame, and a
    0-based principal point through kf_set_intrinsics_ex gives the reference's K."""
    seq, depths = small_seq
    a = make_handle(seq)
    g = seq.cfg.grid
    b = kf.Handle(kf.make_config(height=a.H, width=a.W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size))
    K = seq.K
    b.set_intrinsics(K[0, 0], K[1, 1], np.float32(K[0, 2] - 1), np.float32(K[1, 2] - 1), one_based=False)
    assert np.array_equal(a.intrinsics(), b.intrinsics())
    a.initial_processing(depths[0])
    b.process_frame(depths[0], is_first=True)
    for k in range(1, len(depths)):
        a.incoming_frame(depths[k])
        b.process_frame(depths[k], is_first=False)
        assert np.array_equal(a.pose().view(np.uint32), b.pose().view(np.uint32)), k
    assert np.array_equal(a.predicted().view(np.uint32), b.predicted().view(np.uint32))
    a.close()
    b.close()


def test_invalid_arguments(small_seq):
    seq, _ = small_seq
    h = make_handle(seq)
    with pytest.raises(kf.KinfuError):
        h.set_pose(np.full((4, 4), np.nan, np.float32))
    with pytest.raises(kf.KinfuError):
        h.set_intrinsics(0.0, 525.0, 320.0, 240.0)
    with pytest.raises(ValueError):
        h.incoming_frame(np.zeros((3, 3), np.uint16))


def test_empty_depth_frame(small_seq):
    """An all-zero frame: nothing is integrated or hit, ICP finds no correspondences and
    the pose stays (reference behaviour: cv::Cholesky fails on A = 0, b = 0)."""
    seq, depths = small_seq
    h = make_handle(seq)
    h.initial_processing(depths[0])
    T0 = h.pose()
    zero = np.zeros_like(depths[0])
    h.incoming_frame(zero)
    assert np.array_equal(h.pose(), T0)
    nc, ok = h.icp_stats(10)
    assert np.all(nc == 0) and np.all(ok == 0)
    assert np.all(h.ray_casting() == -1)
