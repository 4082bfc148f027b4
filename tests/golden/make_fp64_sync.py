"""Regenerate tests/golden/fp64_c1_sync.npz -- the FP64 oracle's state at a few frames of
the benchmark sequence, for the benchmark's frame-synced accuracy of the precision form.

For each stored frame k: the FP64 oracle's pose after frame k-1 (poses_prev, double),
its surface prediction after frame k-1 rounded to float (pred_prev: the six 480x640
planes x, y, z, nx, ny, nz, world mm) and its pose after frame k (poses, double).  The
benchmark sets the precision form's handle to pose_prev and pred_prev, runs frame k and
compares the pose with poses[k] -- the same measure as tests/test_precision_synced.py
(mode "icp"), which runs the FP64 oracle live over all 48 frames; the fixture carries
only these frames because the benchmark may not run the oracle.  Also stored: the float
oracle's error (the reference's own arithmetic) from the same state, for comparison.

Workload c1: 640x480 depth into the 360x360x300 grid at 10 mm, the first 48 frames of
its seeded synthetic sequence (the benchmark's frame order starts with them).

    python tests/golden/make_fp64_sync.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

SYNC_FRAMES = (12, 24, 36)


def main() -> None:
    from kinect_fusion_slam_gb300 import scene
    from oracle.pyoracle import GridSpec, Oracle
    from precision_sync import pose_err

    cfg = scene.config("c1")
    n = max(SYNC_FRAMES) + 1
    seq = scene.sequence(cfg, frames=48)
    depths = seq.depths(n)
    g = cfg.grid
    gs = GridSpec(tuple(g.dims), tuple(g.start), float(g.voxel_size), g.truncated_distance, g.sdf_minimum,
                  g.sdf_maximum)
    H, W = depths.shape[1:]
    o = Oracle()
    K = seq.K
    Ki = o.inv3(K)
    p64 = o.pipeline64(H, W, gs, K)
    p64.initial(depths[0])
    prev, pred, poses, float_err = [], [], [], []
    for k in range(1, n):
        T64p = p64.pose.copy()
        P64 = p64.prediction().astype(np.float32)
        p64.incoming(depths[k])
        if k in SYNC_FRAMES:
            prev.append(T64p)
            pred.append(P64)
            poses.append(p64.pose.copy())
            dk = o.depth_ingest(depths[k])
            v5, mask = o.vertex_normal(dk, Ki)
            cur6 = np.stack([v5[0], v5[1], dk, v5[2], v5[3], v5[4]])
            Tf, _ = o.estimate_pose(K, T64p.astype(np.float32), cur6, mask, P64, iters=10)
            float_err.append(pose_err(Tf, poses[-1]))
    p64.close()
    np.savez_compressed(HERE / "fp64_c1_sync.npz", frames=np.array(SYNC_FRAMES, np.int32),
                        poses_prev=np.array(prev), pred_prev=np.array(pred), poses=np.array(poses),
                        float_err=np.array(float_err))
    print("written; float oracle synced error (mm, mrad):", np.array(float_err).round(4).tolist())


if __name__ == "__main__":
    main()
