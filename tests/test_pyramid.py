"""ICP with a 3-level pyramid (10/5/4 iterations, finest first).

The reference tracks at full resolution only (sensor_pose_estimation.cu:339); the
pyramid is a new feature.  Its levels reuse the plain form's kernels (vertex/normal
map, association, the reference-order reduction and the float Cholesky), so the GPU
pyramid is held bit for bit to the float oracle running the same pyramid
(oracle/kf_oracle.cpp: kfo_pyramid_depth, kfo_level_intrinsics, kfo_set_pyramid).
"""
import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from conftest import grid_spec


def test_pyramid_depth_block_average():
    from oracle.pyoracle import Oracle

    o = Oracle()
    d = np.array([[1000, 1010, 0, 0],
                  [1020, 2000, 0, 1500],
                  [0, 0, 700, 0],
                  [0, 0, 0, 0]], np.float32)
    c = o.pyramid_depth(d, band=90.0)
    # 2000 is outside the band around the block's first depth (1000); zeros are skipped
    assert c[0, 0] == np.float32((1000 + 1010 + 1020) / 3)
    assert c[0, 1] == 1500 and c[1, 0] == 0 and c[1, 1] == 700


def test_level_intrinsics():
    from oracle.pyoracle import Oracle

    K = np.array([[525.0, 0, 320.5], [0, 525.0, 240.5], [0, 0, 1]], np.float32)
    K2 = Oracle().level_intrinsics(K, 2)
    # pixel centres of 4x4 blocks: (c - 1/2) / 4 + 1/2 (1-based)
    assert np.allclose(K2, [[131.25, 0, 80.5], [0, 131.25, 60.5], [0, 0, 1]])


@pytest.mark.gpu
def test_pyramid_pipeline_bit_exact_with_oracle(oracle, small_seq):
    seq, depths = small_seq
    H, W = depths.shape[1:]
    g = seq.cfg.grid
    h = kf.Handle(kf.make_config(height=H, width=W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size,
                                 icp_levels=3, icp_iterations=(10, 5, 4)))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    p = oracle.pipeline(H, W, grid_spec(g), K)
    p.set_pyramid(3, [10, 5, 4], band=90.0)
    h.initial_processing(depths[0])
    p.initial(depths[0])
    for k in range(1, 4):
        h.incoming_frame(depths[k])
        p.incoming(depths[k])
        assert np.array_equal(h.pose().view(np.uint32), p.pose.view(np.uint32)), f"frame {k}"
    assert h.kernels_per_frame() == 1 + 3 * 2 + 2 * 19 + 5
    nc, _ = h.icp_stats()
    assert len(nc) == 19 and nc[-1] > 100
    t, w = h.volume()
    to, wo = p.volume()
    assert np.array_equal(np.isnan(w), np.isnan(wo))
    assert np.array_equal(t[~np.isnan(t)].view(np.uint32), to[~np.isnan(to)].view(np.uint32))


@pytest.mark.gpu
def test_precision_form_pyramid_tracks_like_the_plain_pyramid(oracle, small_seq):
    """The precision form's one-pass ICP (fused association, exact fixed-point sums,
    FP64 solve) on the same 3-level pyramid: every level's passes find correspondences,
    and over three tracked frames its distance from the sequence's true poses stays
    within the float pyramid's own plus a millimetre (the tracker turns last-bit
    differences into millimetres within a few frames, so the two forms are compared
    through the ground truth rather than with each other)."""
    seq, depths = small_seq
    H, W = depths.shape[1:]
    g = seq.cfg.grid
    h = kf.Handle(kf.make_config(height=H, width=W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size,
                                 icp_levels=3, icp_iterations=(10, 5, 4), tsdf_storage=kf.KF_TSDF_F16,
                                 solve_mode=kf.KF_SOLVE_PRECISE, icp_reduction=kf.KF_REDUCE_TREE))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    p = oracle.pipeline(H, W, grid_spec(g), K)
    p.set_pyramid(3, [10, 5, 4], band=90.0)
    h.initial_processing(depths[0])
    p.initial(depths[0])
    for k in range(1, 4):
        h.incoming_frame(depths[k])
        p.incoming(depths[k])
        gt = seq.poses[k].astype(np.float64)
        eg = np.linalg.norm(h.pose().astype(np.float64)[:3, 3] - gt[:3, 3])
        eo = np.linalg.norm(p.pose.astype(np.float64)[:3, 3] - gt[:3, 3])
        assert eg <= eo + 1.0 + 0.5 * eo, (k, eg, eo)
    assert h.kernels_per_frame() == 1 + 3 * 2 + 19 + 5
    nc, _ = h.icp_stats()
    assert len(nc) == 19 and min(nc) > 10
