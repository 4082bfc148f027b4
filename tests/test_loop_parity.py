"""GPU parity of the whole frame loop (KinfuPipeline::InitialProcessing /
IncomingFrameProcessing, kinfu_pipeline.cpp:91-193) against the CPU oracle's loop,
free-running on both sides:

* c1, the bench's workload (640x480 into 360x360x300 @ 10 mm), plain form;
* the reference's own recorded Kinect frames dep0025-0027 (system_utility.cpp:58-68),
  whose holes, edges and noise the synthetic room does not have;
* the bilateral stage switched on at the reference's commented-out call site
  (kinfu_pipeline.cpp:141-145, bilateral_filtering.cu:3-47);
* the error path of the bounded device waits (kf_set_wait_limit), made to run out by a
  host setting: no fault, trap or hang is involved.

Gates: poses bit for bit at every frame, the integrated voxel set and weight counts bit
for bit, TSDF values within 1e-6, ray-cast hit voxel indices bit for bit.
"""
import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from conftest import grid_spec, real_frame
from test_gpu_parity import POINT_TOL_MM, assert_volume_parity, make_handle

pytestmark = pytest.mark.gpu

BILATERAL_TOL_MM = 1e-2  # CUDA's expf against glibc's, through the 7x7 weights


def _free_run(oracle, h, o, depths, check_hits_every=1):
    h.initial_processing(depths[0])
    o.initial(depths[0])
    for k in range(1, len(depths)):
        h.incoming_frame(depths[k])
        o.incoming(depths[k])
        Tg, To = h.pose(), o.pose
        assert np.array_equal(Tg.view(np.uint32), To.view(np.uint32)), f"frame {k}: pose bits differ\n{Tg}\n{To}"
        if k % check_hits_every == 0 or k == len(depths) - 1:
            _, hit_o = o.prediction()
            hit_g = h.ray_casting()
            assert np.array_equal(hit_g, hit_o), f"frame {k}: {int((hit_g != hit_o).sum())} hit indices differ"


def test_pipeline_free_running_c1(oracle):
    """c1 free-running for 12 frames (the first InitialProcessing and 11 incoming frames
    with 10 ICP iterations each): the GPU's plain form and the float oracle produce the
    same pose at every frame, the same hit indices, and after the last frame the same
    volume."""
    from kinect_fusion_slam_gb300 import scene

    n = 12
    seq = scene.sequence("c1", frames=n)
    depths = seq.depths(n)
    gs = grid_spec(seq.cfg.grid)
    h = make_handle(seq)
    o = oracle.pipeline(480, 640, gs, seq.K)
    _free_run(oracle, h, o, depths, check_hits_every=3)
    tg, wg = h.volume()
    to, wo = o.volume()
    assert_volume_parity(tg, wg, to, wo)
    assert int((~np.isnan(wo)).sum()) > 1_000_000
    assert int(np.nanmax(wo)) == n  # voxels seen in every frame
    pred_o, hit_o = o.prediction()
    m = hit_o >= 0
    assert np.abs(h.predicted()[:3][:, m] - pred_o[:3][:, m]).max() <= POINT_TOL_MM
    h.close()
    o.close()


def test_pipeline_real_frames():
    """The reference's recorded frames 25-27 at its own intrinsics and default grid
    (kinfu_pipeline.cpp:14-58): InitialProcessing on frame 25, then frames 26 and 27,
    GPU against the float oracle, bit for bit."""
    from oracle.pyoracle import GridSpec, Oracle, reference_K

    oracle = Oracle()
    depths = [real_frame(i) for i in (25, 26, 27)]
    assert all(d.shape == (480, 640) for d in depths)
    K = reference_K()
    h = kf.Handle(kf.make_config())
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    o = oracle.pipeline(480, 640, GridSpec(), K)
    _free_run(oracle, h, o, depths)
    tg, wg = h.volume()
    to, wo = o.volume()
    assert_volume_parity(tg, wg, to, wo)
    _, hit_o = o.prediction()
    # recorded depth: ~200 k of 307 200 rays reach a surface (197 354 on frame 25)
    assert int((hit_o >= 0).sum()) > 150_000
    nc, _ = h.icp_stats(10)
    assert nc[0] > 100_000
    h.close()
    o.close()


def test_bilateral_stage_in_loop(oracle, c0_seq):
    """kf_config.bilateral = 1: the 7x7 bilateral filter runs after the vertex map at the
    reference's commented-out call site, and its output replaces the depth that ICP (as
    the vertices' z), integration and the ray cast read.  Free-running on c0 (640x480,
    180x180x150 @ 20 mm): each frame's filtered depth is within 1e-2 mm of the oracle's
    filter (CUDA's expf against glibc's), and the oracle's loop, given the GPU's filtered
    depth, reproduces every pose, weight and hit index bit for bit."""
    seq, depths = c0_seq
    depths = depths[:8]
    gs = grid_spec(seq.cfg.grid)
    h = make_handle(seq, bilateral=1)
    o = oracle.pipeline(480, 640, gs, seq.K)
    o.set_bilateral(True, radius=3, sigma_d=4.5, sigma_r=30.0)
    r, sd = 3, 4.5
    yy, xx = np.mgrid[-r:r + 1, -r:r + 1].astype(np.float32)
    spatial = np.exp((-(xx * xx + yy * yy) / np.float32(2 * sd * sd)).astype(np.float64)).astype(np.float32)
    h.initial_processing(depths[0])
    o.initial(depths[0])
    worst = 0.0
    for k in range(1, len(depths)):
        h.incoming_frame(depths[k])
        filtered_g = h.depth()
        filtered_o = oracle.bilateral(oracle.depth_ingest(depths[k]), spatial, r, 30.0)
        worst = max(worst, float(np.abs(filtered_g - filtered_o).max()))
        assert np.abs(filtered_g - filtered_o).max() <= BILATERAL_TOL_MM
        o.incoming(depths[k], filtered=filtered_g)
        assert np.array_equal(h.pose().view(np.uint32), o.pose.view(np.uint32)), f"frame {k}: pose bits differ"
        _, hit_o = o.prediction()
        assert np.array_equal(h.ray_casting(), hit_o), f"frame {k}: hit indices differ"
    tg, wg = h.volume()
    to, wo = o.volume()
    assert_volume_parity(tg, wg, to, wo)
    # the stage changes the result: without it the same frames give another trajectory
    h2 = make_handle(seq)
    h2.initial_processing(depths[0])
    for k in range(1, len(depths)):
        h2.incoming_frame(depths[k])
    assert not np.array_equal(h2.pose(), h.pose())
    print(f"bilateral in the loop: worst filtered-depth difference {worst:.2e} mm")
    h.close()
    h2.close()
    o.close()


def test_bounded_wait_error_path(small_seq):
    """The plain form's in-order reduction streams the ICP group sums through shared
    memory with bulk copies and waits for each with a bounded poll.  With the poll limit
    set to 0 every such wait gives up at once: the kernel sets the handle's error flag,
    waits for its copies in flight at the default limit, and returns without changing
    the pose.  kf_get_pose reports KF_ERR_CUDA with the unchanged pose; kf_icp_associate
    reports the error instead of sums; after the default limit is restored the next
    frame runs normally and matches a handle that never saw the error."""
    seq, depths = small_seq
    h = make_handle(seq)
    ref = make_handle(seq)
    for x in (h, ref):
        x.initial_processing(depths[0])
        x.incoming_frame(depths[1])
    T_before = h.pose()
    assert np.array_equal(T_before, ref.pose())
    h.set_wait_limit(0)
    h.incoming_frame(depths[2])
    with pytest.raises(kf.KinfuError) as ei:
        h.pose()
    assert ei.value.status == kf.KF_ERR_CUDA
    # every iteration gave up before its update: the pose is the one before the frame
    T_err = np.zeros((4, 4), np.float32)
    assert h.lib.kf_get_pose(h.h, T_err) == kf.KF_OK  # the flag was cleared by the report
    assert np.array_equal(T_err, T_before)
    F = np.eye(4, dtype=np.float32)
    with pytest.raises(kf.KinfuError):
        h.icp_associate(F, T_before)
    h.set_wait_limit(-1)
    # back to normal: replay the failed frame from the same start on both handles
    for x in (h, ref):
        x.reset()
        x.initial_processing(depths[0])
        x.incoming_frame(depths[1])
        x.incoming_frame(depths[2])
    assert np.array_equal(h.pose().view(np.uint32), ref.pose().view(np.uint32))
    h.close()
    ref.close()
