"""The frame calls' host-side overlap: a pinned host frame is staged one frame ahead on a
copy stream into one of two raw buffers, and kf_get_pose right after a frame call reads
the pose once the ICP has finished, while integration and the ray cast still run.

Neither may change a result: the same frames through the device-input path, the pinned
path (reading the pose after every frame, or running ahead several frames between
reads), the pageable path, and with other calls between a frame and its pose, give the
same poses and the same predicted surface, bit for bit."""
import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf

pytestmark = pytest.mark.gpu


PRECISION = dict(tsdf_storage=kf.KF_TSDF_F16, solve_mode=kf.KF_SOLVE_PRECISE, icp_reduction=kf.KF_REDUCE_TREE)


def _handle(seq, H, W, **extra):
    g = seq.cfg.grid
    h = kf.Handle(
        kf.make_config(height=H, width=W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size, **extra))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    return h


def _run(seq, depths, mode, **extra):
    import torch

    H, W = depths.shape[1:]
    h = _handle(seq, H, W, **extra)
    n = len(depths)
    fb = H * W * 2
    pinned = torch.from_numpy(depths.view(np.int16)).pin_memory()
    dev = pinned.cuda()
    poses = []
    for k in range(n):
        if mode == "device":
            (h.initial_processing_device if k == 0 else h.incoming_frame_device)(dev.data_ptr() + k * fb)
        elif mode in ("pinned", "pinned_ahead", "pinned_interleaved"):
            (h.initial_processing_ptr if k == 0 else h.incoming_frame_ptr)(pinned.data_ptr() + k * fb)
        else:
            (h.initial_processing if k == 0 else h.incoming_frame)(depths[k])
        if mode == "pinned_interleaved":
            h.intrinsics()  # another call between the frame and its pose: the full synchronisation
        if mode != "pinned_ahead" or k == n - 1:
            poses.append(h.pose())
    pred = h.predicted()
    h.close()
    return poses, pred


def _same(a, b):
    return np.array_equal(np.asarray(a).view(np.uint32), np.asarray(b).view(np.uint32))


@pytest.mark.parametrize("form", ["plain", "precision"])
def test_pinned_pageable_and_device_frames_agree(small_seq, form):
    """Every input path, with and without the per-frame CUDA graphs, against the graph
    device-input run.  The precision form's sums are exact fixed-point accumulations, so
    its results do not depend on the order the blocks finish in either."""
    seq, depths = small_seq
    depths = np.concatenate([depths, depths[::-1][1:]])  # 7 frames: forwards and back
    extra = PRECISION if form == "precision" else {}
    ref_poses, ref_pred = _run(seq, depths, "device", **extra)
    for graphs in (1, 0):
        for mode in ("device", "pinned", "pageable", "pinned_interleaved"):
            if graphs and mode == "device":
                continue
            poses, pred = _run(seq, depths, mode, use_graphs=graphs, **extra)
            assert all(_same(a, b) for a, b in zip(poses, ref_poses)), (mode, graphs)
            assert _same(pred, ref_pred), (mode, graphs)
        poses, pred = _run(seq, depths, "pinned_ahead", use_graphs=graphs, **extra)
        assert _same(poses[-1], ref_poses[-1]), graphs
        assert _same(pred, ref_pred), graphs
