"""Pins the CPU oracle to the reference itself: the reference's kernel bodies compiled
for the CPU (oracle/_ref, built by oracle/build.py) and the oracle restatement must
agree bit for bit -- TSDF and weights, ray-cast outputs and hit voxels, vertex maps,
ICP sums, and the poses of whole frame sequences."""
import numpy as np
import pytest

from conftest import grid_spec, real_frame


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_vertex_normal(oracle, reference, small_seq):
    seq, depths = small_seq
    Ki = oracle.inv3(seq.K)
    for d in depths:
        dep = oracle.depth_ingest(d)
        vo, mo = oracle.vertex_normal(dep, Ki)
        vr, mr = reference.vertex_normal(dep, Ki)
        assert np.array_equal(mo, mr)
        assert np.array_equal(bits(vo), bits(vr))


def test_integrate_and_raycast(oracle, reference, small_seq):
    seq, depths = small_seq
    gs = grid_spec(seq.cfg.grid)
    K = seq.K
    Ki = oracle.inv3(K)
    vols = {}
    for name, impl in (("o", oracle), ("r", reference)):
        t = np.full(gs.nvox, np.nan, np.float32)
        w = np.full(gs.nvox, np.nan, np.float32)
        for n, k in enumerate(range(3)):
            T = seq.poses[k].astype(np.float32)
            impl.integrate(gs, oracle.depth_ingest(depths[k]), K, Ki, T, oracle.inv4(T), t, w, first=(n == 0))
        vols[name] = (t, w)
    assert np.array_equal(bits(vols["o"][0]), bits(vols["r"][0]))
    assert np.array_equal(bits(vols["o"][1]), bits(vols["r"][1]))
    T = seq.poses[3].astype(np.float32)
    d = oracle.depth_ingest(depths[3])
    po, ho = oracle.raycast(gs, d, Ki, T, vols["o"][0])
    pr, hr = reference.raycast(gs, d, Ki, T, vols["r"][0])
    assert np.array_equal(ho, hr)
    assert (ho >= 0).sum() > 300
    assert np.array_equal(bits(po), bits(pr))


def test_icp_sums_and_pose(oracle, reference, small_seq):
    seq, depths = small_seq
    gs = grid_spec(seq.cfg.grid)
    K = seq.K
    Ki = oracle.inv3(K)
    t = np.full(gs.nvox, np.nan, np.float32)
    w = np.full(gs.nvox, np.nan, np.float32)
    T0 = seq.poses[0].astype(np.float32)
    d0 = oracle.depth_ingest(depths[0])
    oracle.integrate(gs, d0, K, Ki, T0, oracle.inv4(T0), t, w, first=True)
    pred6, _ = oracle.raycast(gs, d0, Ki, T0, t)
    d1 = oracle.depth_ingest(depths[1])
    v5, mask = oracle.vertex_normal(d1, Ki)
    cur6 = np.stack([v5[0], v5[1], d1, v5[2], v5[3], v5[4]])
    F = oracle.matmul4(oracle.inv4(T0), T0)
    n_o, s_o, pair_o = oracle.icp_associate(K, F, T0, cur6, mask, pred6)
    n_r, s_r, flag_r = reference.icp_associate(K, F, T0, cur6, mask, pred6)
    assert n_o == n_r and n_o > 100
    assert np.array_equal((pair_o >= 0).astype(np.int32), flag_r)
    assert np.array_equal(bits(s_o), bits(s_r))
    To, log_o = oracle.estimate_pose(K, T0, cur6, mask, pred6, iters=10)
    Tr, log_r = reference.estimate_pose(K, T0, cur6, mask, pred6, iters=10)
    assert np.array_equal(bits(log_o["sums"]), bits(log_r["sums"]))
    assert np.array_equal(bits(To), bits(Tr))


def test_pipeline_synthetic(oracle, reference, small_seq):
    seq, depths = small_seq
    gs = grid_spec(seq.cfg.grid)
    H, W = seq.cfg.camera.height, seq.cfg.camera.width
    po = oracle.pipeline(H, W, gs, seq.K)
    pr = reference.pipeline(H, W, gs, seq.K)
    po.initial(depths[0])
    pr.initial(depths[0])
    for k in range(1, len(depths)):
        po.incoming(depths[k])
        pr.incoming(depths[k])
        assert np.array_equal(bits(po.pose), bits(pr.pose))
    to, wo = po.volume()
    tr, wr = pr.volume()
    assert np.array_equal(bits(to), bits(tr)) and np.array_equal(bits(wo), bits(wr))
    o6, ho = po.prediction()
    r6, hr = pr.prediction()
    assert np.array_equal(ho, hr) and np.array_equal(bits(o6), bits(r6))


@pytest.mark.slow
def test_pipeline_real_frames(oracle, reference):
    """The reference's default configuration on its own recorded frames 25..27."""
    from oracle.pyoracle import GridSpec, reference_K

    gs = GridSpec()
    po = oracle.pipeline(480, 640, gs, reference_K())
    pr = reference.pipeline(480, 640, gs, reference_K())
    po.initial(real_frame(25))
    pr.initial(real_frame(25))
    _, hit = po.prediction()
    assert int((hit >= 0).sum()) == 197354  # zero-initialised XY..ZY convention
    for f in (26, 27):
        po.incoming(real_frame(f))
        pr.incoming(real_frame(f))
        assert np.array_equal(bits(po.pose), bits(pr.pose))
    to, wo = po.volume()
    tr, wr = pr.volume()
    assert np.array_equal(bits(to), bits(tr)) and np.array_equal(bits(wo), bits(wr))
    o6, ho = po.prediction()
    r6, hr = pr.prediction()
    assert np.array_equal(ho, hr) and np.array_equal(bits(o6), bits(r6))


def test_bilateral_interior(oracle, reference, small_seq):
    """The oracle tightens the reference's out-of-image bound; away from that border
    row/column both agree bit for bit."""
    seq, depths = small_seq
    d = oracle.depth_ingest(depths[0])
    r = 3
    yy, xx = np.mgrid[-r:r + 1, -r:r + 1].astype(np.float32)
    spatial = np.exp(-(xx * xx + yy * yy) / np.float32(2 * 4.5 * 4.5)).astype(np.float32)
    bo = oracle.bilateral(d, spatial, r, 30.0)
    br = reference.bilateral(d, spatial, r, 30.0)
    H, W = d.shape
    assert np.array_equal(bits(bo[: H - r, : W - r]), bits(br[: H - r, : W - r]))
    # the tightened bound leaves row H-1-r+1 and column W-1-r+1 at zero
    assert np.all(bo[H - r, :] == 0) and np.all(bo[:, W - r] == 0)


def test_reference_integration_skips_last_voxel(oracle, reference):
    """projective_tsdf.cu:14 compares the int thread index with a float voxel count, so
    at 360x360x300 the last voxel is never integrated; the oracle reproduces it."""
    from oracle.pyoracle import GridSpec

    gs = GridSpec()
    H, W = 8, 8
    # one depth pixel seen straight on at the far corner is enough to exercise the guard:
    # integrate with a pose that puts the last voxel in view and compare
    K = np.array([[4.0, 0, 4.5], [0, 4.0, 4.5], [0, 0, 1]], np.float32)
    Ki = oracle.inv3(K)
    T = np.eye(4, dtype=np.float32)
    T[:3, 3] = [1595.0, 1595.0, 1400.0]
    depth = np.full((H, W), 400.0, np.float32)
    to = np.full(gs.nvox, np.nan, np.float32)
    wo = np.full(gs.nvox, np.nan, np.float32)
    tr, wr = to.copy(), wo.copy()
    oracle.integrate(gs, depth, K, Ki, T, oracle.inv4(T), to, wo, first=True)
    reference.integrate(gs, depth, K, Ki, T, oracle.inv4(T), tr, wr, first=True)
    assert np.array_equal(bits(to), bits(tr)) and np.array_equal(bits(wo), bits(wr))
    assert np.isnan(wo[-1])


def test_integration_wide_angle_behind_camera(oracle, reference, small_seq):
    """With a 30 px focal length on 160 x 120 the reference's in-front axis, built from the
    swapped principal point (projective_tsdf.cu:57-73), tilts far enough that voxels
    behind the camera pass it and, projecting mirrored into the image, are updated (the
    GPU's box marks cover them).  The oracle reproduces the reference bit for bit here,
    with near, infinite, 1e30 and NaN depths among ordinary ones."""
    seq, _ = small_seq
    gs = grid_spec(seq.cfg.grid)
    H, W = seq.cfg.camera.height, seq.cfg.camera.width
    K = np.array([[30.0, 0.0, W / 2 + 0.5], [0.0, 30.0, H / 2 + 0.5], [0.0, 0.0, 1.0]], np.float32)
    Ki = oracle.inv3(K)
    rng = np.random.default_rng(17)
    c, s = np.cos(0.3), np.sin(0.3)
    T = np.array([[c, 0, s, 200.0], [0, 1, 0, -150.0], [-s, 0, c, -300.0], [0, 0, 0, 1]], np.float32)
    yy, xx = np.mgrid[0:H, 0:W]
    depth = (400.0 + 300.0 * np.sin(xx / 9.0) * np.cos(yy / 7.0)).astype(np.float32)
    near = rng.random((H, W)) < 0.1
    depth[near] = rng.uniform(50.0, 150.0, int(near.sum())).astype(np.float32)
    for value, frac in [(0.0, 0.1), (np.inf, 0.01), (1e30, 0.01), (np.nan, 0.01)]:
        depth[rng.random((H, W)) < frac] = value
    vols = {}
    for name, impl in (("o", oracle), ("r", reference)):
        t = np.full(gs.nvox, np.nan, np.float32)
        w = np.full(gs.nvox, np.nan, np.float32)
        impl.integrate(gs, depth, K, Ki, T, oracle.inv4(T), t, w, first=True)
        vols[name] = (t, w)
    assert np.array_equal(bits(vols["o"][0]), bits(vols["r"][0]))
    assert np.array_equal(bits(vols["o"][1]), bits(vols["r"][1]))
    # updated voxels behind the camera (z-fastest index: ((x * dy) + y) * dz + z)
    dims = gs.dims
    upd = np.flatnonzero(~np.isnan(vols["r"][1]))
    ijk = np.stack([upd // (dims[1] * dims[2]), (upd // dims[2]) % dims[1], upd % dims[2]], 1)
    centres = (ijk + np.asarray(gs.start) + 0.5) * gs.voxel_size
    lz = (centres - T[:3, 3].astype(np.float64)) @ T[:3, 2].astype(np.float64)
    assert np.count_nonzero(lz < 0) > 1000
