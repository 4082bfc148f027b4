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


def _handle(seq, H, W):
    g = seq.cfg.grid
    h = kf.Handle(kf.make_config(height=H, width=W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    return h


def _run(seq, depths, mode):
    import torch

    H, W = depths.shape[1:]
    h = _handle(seq, H, W)
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


def test_pinned_pageable_and_device_frames_agree(small_seq):
    seq, depths = small_seq
    depths = np.concatenate([depths, depths[::-1][1:]])  # 7 frames: forwards and back
    ref_poses, ref_pred = _run(seq, depths, "device")
    for mode in ("pinned", "pageable", "pinned_interleaved"):
        poses, pred = _run(seq, depths, mode)
        assert all(np.array_equal(a.view(np.uint32), b.view(np.uint32)) for a, b in zip(poses, ref_poses)), mode
        assert np.array_equal(pred.view(np.uint32), ref_pred.view(np.uint32)), mode
    poses, pred = _run(seq, depths, "pinned_ahead")
    assert np.array_equal(poses[-1].view(np.uint32), ref_poses[-1].view(np.uint32))
    assert np.array_equal(pred.view(np.uint32), ref_pred.view(np.uint32))
