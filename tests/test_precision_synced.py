"""The precision form's <= 1 mm bar against the FP64 oracle, frame by frame.

The FP16-TSDF form (FP16 value + weight storage, FP32 association, compensated sums,
FP64 solve and pose composition) is to track within 1 mm of the FP64 oracle.  A
free-running comparison cannot show that for any implementation of this tracker: it
amplifies last-bit differences into centimetres within a few frames (the reference's
own float arithmetic is 22 mm from the FP64 run after 48 frames of c1).  So each frame
starts from the FP64 oracle's state and the step it takes is compared with the FP64
oracle's own step (tests/precision_sync.py), over c1's first 48 frames and c2's first 12:

* mode "icp": the FP64 oracle's pose and surface prediction -- the error of the form's
  ICP arithmetic (sensor_pose_estimation.cu:339-429);
* mode "frame": the FP64 oracle's pose and volume, stored as the form's FP16 pair and ray
  cast by the GPU -- adds the FP16 TSDF and the float ray cast (voxel_traversal.cu).

Both must stay within 1 mm at every frame.  The float oracle's synced error (the
reference's own arithmetic) is printed beside them.
"""
import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from precision_sync import summary, synced_errors

pytestmark = pytest.mark.gpu

SYNC_TOL_MM = 1.0    # the precision form's bar: <= 1 mm of trajectory (translation) against FP64
# a guard on the rotation, which the bar does not state: the FP16 volume's ray cast has
# moved one frame's rotation by 1.04 mrad (c1, mode "frame"; 0.34 mrad from the ICP alone)
SYNC_TOL_MRAD = 2.0


def precision_handle(seq):
    g, cam = seq.cfg.grid, seq.cfg.camera
    h = kf.Handle(kf.make_config(height=cam.height, width=cam.width, dims=g.dims, grid_start=g.start,
                                 voxel_size=g.voxel_size, tsdf_storage=kf.KF_TSDF_F16,
                                 icp_reduction=kf.KF_REDUCE_TREE, solve_mode=kf.KF_SOLVE_PRECISE))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    return h


@pytest.mark.parametrize("name,frames", [("c1", 48), ("c2", 12)])
def test_precision_form_synced_to_fp64(oracle, name, frames):
    from kinect_fusion_slam_gb300 import scene

    seq = scene.sequence(name, frames=frames)
    depths = seq.depths(frames)
    h = precision_handle(seq)
    err = synced_errors(oracle, h, seq, depths)
    h.close()
    s = {m: summary(e) for m, e in err.items()}
    for m, v in s.items():
        print(f"{name} synced to FP64, {m:5s}: rms {v['rms_mm']:.4f} mm, max {v['max_mm']:.4f} mm, "
              f"rms {v['rms_mrad']:.5f} mrad, max {v['max_mrad']:.5f} mrad over {v['frames']} frames")
    for m in ("icp", "frame"):
        assert s[m]["max_mm"] <= SYNC_TOL_MM, (m, s[m])
        assert s[m]["max_mrad"] <= SYNC_TOL_MRAD, (m, s[m])


def test_plain_form_synced_equals_float_oracle(oracle):
    """The plain form's synced step is the float oracle's bit for bit (same pose and
    prediction in, same ICP arithmetic), so their errors against FP64 are identical."""
    from kinect_fusion_slam_gb300 import scene

    seq = scene.sequence("c1", frames=6)
    depths = seq.depths(6)
    g, cam = seq.cfg.grid, seq.cfg.camera
    h = kf.Handle(kf.make_config(height=cam.height, width=cam.width, dims=g.dims, grid_start=g.start,
                                 voxel_size=g.voxel_size))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    err = synced_errors(oracle, h, seq, depths, modes=("icp",))
    h.close()
    assert np.array_equal(err["icp"], err["float"])
