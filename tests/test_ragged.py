"""Ragged sizes.  The image is 157 x 117 = 18 369 pixels: 287 ICP groups of 64 and one
pixel, and sides that are not multiples of the ray cast's 8 x 4 tiles.  The grid is
173 x 161 x 147 voxels, no side a multiple of integration's 32 x 8 x 8 boxes.  The
pyramid case uses 156 x 116 (divisible by 4, as three levels need), whose levels hold
18 096, 4 524 and 1 131 pixels.

The plain form runs free beside the float oracle and must agree with it bit for bit:
poses, voxels, weights and hit indices.  The precision form must track like the float
oracle, and a batch holding the ragged scene beside a regular one must give each scene
the results it gets alone."""
import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from conftest import grid_spec
from kinect_fusion_slam_gb300 import scene
from test_gpu_parity import POINT_TOL_MM, assert_volume_parity

pytestmark = pytest.mark.gpu

FRAMES = 6
PRECISION = dict(tsdf_storage=kf.KF_TSDF_F16, solve_mode=kf.KF_SOLVE_PRECISE, icp_reduction=kf.KF_REDUCE_TREE)


def _seq(W, H):
    # a quarter-size Kinect camera with its principal point at the image centre
    cam = scene.Camera(W, H, 525.0 * 0.245, 525.0 * 0.245, (W - 1) / 2, (H - 1) / 2)
    g = scene.GridConfig((173, 161, 147), 20.0, origin_mm=(-1860.0, -1720.0, -1180.0))
    seq = scene.sequence(scene.SceneConfig(f"ragged{W}x{H}", g, 300, camera=cam, seed=77))
    return seq, seq.depths(FRAMES)


@pytest.fixture(scope="module")
def ragged():
    return _seq(157, 117)


def _config(seq, **kw):
    g, cam = seq.cfg.grid, seq.cfg.camera
    return kf.make_config(height=cam.height, width=cam.width, dims=g.dims, grid_start=g.start,
                          voxel_size=g.voxel_size, **kw)


def _handle(seq, **kw):
    h = kf.Handle(_config(seq, **kw))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    return h


def _free_run(oracle, seq, depths, levels):
    H, W = depths.shape[1:]
    it = (10, 5, 4)[:levels]
    h = _handle(seq, icp_levels=levels, icp_iterations=it)
    p = oracle.pipeline(H, W, grid_spec(seq.cfg.grid), seq.K)
    if levels > 1:
        p.set_pyramid(levels, list(it), band=90.0)
    h.initial_processing(depths[0])
    p.initial(depths[0])
    for k in range(1, len(depths)):
        h.incoming_frame(depths[k])
        p.incoming(depths[k])
        assert np.array_equal(h.pose().view(np.uint32), p.pose.view(np.uint32)), f"frame {k}"
    nc, _ = h.icp_stats()
    assert len(nc) == sum(it) and min(nc) > 10
    tg, wg = h.volume()
    to, wo = p.volume()
    assert_volume_parity(tg, wg, to, wo)
    pred_o, hit_o = p.prediction()
    assert np.array_equal(h.ray_casting(), hit_o) and int((hit_o >= 0).sum()) > H * W // 2
    pred_g, m = h.predicted(), hit_o >= 0
    assert np.abs(pred_g[:3][:, m] - pred_o[:3][:, m]).max() <= POINT_TOL_MM
    assert np.array_equal(np.isnan(pred_g), np.isnan(pred_o)) and np.all(pred_g[:, ~m] == 0)
    h.close()


def test_ragged_plain_form_bit_exact(oracle, ragged):
    seq, depths = ragged
    _free_run(oracle, seq, depths, 1)


def test_ragged_pyramid_bit_exact(oracle):
    seq, depths = _seq(156, 116)
    _free_run(oracle, seq, depths, 3)


def test_ragged_precision_form_tracks(oracle, ragged):
    """The precision form against the sequence's true poses, within the float oracle's
    own distance from them plus a millimetre (the tracker turns last-bit differences
    into millimetres within a few frames, so the forms are compared through the ground
    truth); every ICP pass finds correspondences."""
    seq, depths = ragged
    H, W = depths.shape[1:]
    h = _handle(seq, **PRECISION)
    p = oracle.pipeline(H, W, grid_spec(seq.cfg.grid), seq.K)
    h.initial_processing(depths[0])
    p.initial(depths[0])
    for k in range(1, len(depths)):
        h.incoming_frame(depths[k])
        p.incoming(depths[k])
        gt = seq.poses[k][:3, 3]
        eg = np.linalg.norm(h.pose().astype(np.float64)[:3, 3] - gt)
        eo = np.linalg.norm(p.pose.astype(np.float64)[:3, 3] - gt)
        assert eg <= eo + 1.0 + 0.5 * eo, (k, eg, eo)
        nc, _ = h.icp_stats()
        assert min(nc) > 10
    assert int((h.ray_casting() >= 0).sum()) > H * W // 2
    h.close()


@pytest.mark.parametrize("storage", [kf.KF_TSDF_F32, kf.KF_TSDF_F16])
def test_ragged_scene_in_a_batch(ragged, small_seq, storage):
    """The batching form takes the reference's reduction and solve, with either volume
    storage."""
    torch = pytest.importorskip("torch")
    extra = dict(tsdf_storage=storage)
    data = [ragged, small_seq]
    configs = [_config(seq, **extra) for seq, _ in data]
    b = kf.Batch(configs)
    singles = [kf.Handle(c) for c in configs]
    for (seq, _), hb, hs in zip(data, b.scenes, singles):
        for h in (hb, hs):
            K = seq.K
            h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    n = min(len(d) for _, d in data)
    dev = [torch.from_numpy(np.ascontiguousarray(d[:n]).view(np.int16)).cuda() for _, d in data]
    fb = [c.height * c.width * 2 for c in configs]
    b.initial_processing_device([t.data_ptr() for t in dev])
    for h, t in zip(singles, dev):
        h.initial_processing_device(t.data_ptr())
    for k in range(1, n):
        b.incoming_frame_device([t.data_ptr() + k * m for t, m in zip(dev, fb)])
        for h, t, m in zip(singles, dev, fb):
            h.incoming_frame_device(t.data_ptr() + k * m)
        b.synchronize()
        for i, (hb, hs) in enumerate(zip(b.scenes, singles)):
            assert np.array_equal(hb.pose().view(np.uint32), hs.pose().view(np.uint32)), f"scene {i} frame {k}"
    for hb, hs in zip(b.scenes, singles):
        tb, wb = hb.volume()
        ts, ws = hs.volume()
        assert np.array_equal(tb.view(np.uint32), ts.view(np.uint32))
        assert np.array_equal(wb.view(np.uint32), ws.view(np.uint32))
        assert np.array_equal(hb.predicted().view(np.uint32), hs.predicted().view(np.uint32))
    for h in singles:
        h.close()
    b.close()
