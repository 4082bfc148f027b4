"""The batching form: uneven scenes, one launch per stage, one CUDA graph per frame.

Each scene of a batch runs the single-scene kernels' device code, so its poses, volume
and prediction must be bit-identical to the same scene run alone on its own handle --
with the default launch shapes and after the autotuner has picked others.
"""
import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from kinect_fusion_slam_gb300 import scene

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _scenes():
    cams = [scene.Camera().scaled(0.25), scene.Camera().scaled(0.5), scene.Camera().scaled(0.25)]
    grids = [scene.GridConfig((180, 180, 150), 20.0),
             scene.GridConfig((128, 128, 128), 20.0, origin_mm=(-1280.0, -1280.0, -400.0)),
             scene.GridConfig((96, 120, 100), 25.0, origin_mm=(-1200.0, -1500.0, -500.0))]
    out = []
    for i, (cam, g) in enumerate(zip(cams, grids)):
        seq = scene.sequence(scene.SceneConfig(f"b{i}", g, 4, camera=cam, seed=300 + i))
        out.append((seq, seq.depths(4)))
    return out


def _config(seq, depths, levels):
    H, W = depths.shape[1:]
    g = seq.cfg.grid
    return kf.make_config(height=H, width=W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size,
                          icp_levels=levels, icp_iterations=(10, 5, 4)[:levels])


def _intrinsics(h, seq):
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])


@pytest.mark.parametrize("levels,tune,persistent", [(1, False, False), (3, True, False), (1, False, True),
                                                   (3, True, True)])
def test_batch_matches_scenes_run_alone(levels, tune, persistent):
    """persistent: integration and the ICP group pass spread over one fixed grid for all
    scenes (kf_batch_set_forms) instead of one row of blocks per scene."""
    data = _scenes()
    configs = [_config(seq, d, levels) for seq, d in data]
    b = kf.Batch(configs)
    b.set_forms(persistent, persistent)
    singles = [kf.Handle(c) for c in configs]
    for (seq, _), hb, hs in zip(data, b.scenes, singles):
        _intrinsics(hb, seq)
        _intrinsics(hs, seq)
    dev = [torch.from_numpy(d.view(np.int16)).cuda() for _, d in data]
    fb = [s.config.height * s.config.width * 2 for s in singles]
    b.initial_processing_device([t.data_ptr() for t in dev])
    for h, t in zip(singles, dev):
        h.initial_processing_device(t.data_ptr())
    if tune:
        b.synchronize()
        tuning = b.autotune()
        assert tuning[0] in (4, 8, 16) and tuning[1] in (0, 1, 2) and 1 <= tuning[2] <= 4
    assert b.kernels_per_frame() == 1 + 2 * (levels - 1) + 2 * sum((10, 5, 4)[:levels]) + 3
    for k in range(1, 4):
        b.incoming_frame_device([t.data_ptr() + k * n for t, n in zip(dev, fb)])
        for h, t, n in zip(singles, dev, fb):
            h.incoming_frame_device(t.data_ptr() + k * n)
        b.synchronize()
        for i, (hb, hs) in enumerate(zip(b.scenes, singles)):
            assert np.array_equal(hb.pose().view(np.uint32), hs.pose().view(np.uint32)), f"scene {i} frame {k}"
    for hb, hs in zip(b.scenes, singles):
        tb, wb = hb.volume()
        ts, ws = hs.volume()
        assert np.array_equal(tb.view(np.uint32), ts.view(np.uint32))
        assert np.array_equal(wb.view(np.uint32), ws.view(np.uint32))
        assert np.array_equal(hb.predicted().view(np.uint32), hs.predicted().view(np.uint32))
        nc, _ = hb.icp_stats()
        assert nc[-1] > 100
    b.close()


def test_batch_rejects_mixed_schedules():
    c1 = kf.make_config(height=120, width=160, dims=(64, 64, 64))
    c2 = kf.make_config(height=120, width=160, dims=(64, 64, 64), tsdf_storage=kf.KF_TSDF_F16)
    with pytest.raises(kf.KinfuError):
        kf.Batch([c1, c2])
