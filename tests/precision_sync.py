"""Frame-synced accuracy of a tracking form against the FP64 oracle (test helper).

A free-running trajectory of this tracker turns a difference in the last bit into
millimetres within a few frames (the reference's own float arithmetic ends 22 mm from
the FP64 run over 48 frames of c1).  What the arithmetic of one form contributes is the
error of a single frame step taken from the same state.  So at every frame k the GPU
handle starts from the FP64 oracle's state after frame k-1 -- its pose and its surface
prediction (mode "icp"), or its pose and its volume, stored in the handle's TSDF form and
ray cast by the handle (mode "frame") -- runs IncomingFrameProcessing on frame k, and the
resulting pose is compared with the FP64 oracle's own pose after frame k.

The float oracle (the reference's arithmetic, sensor_pose_estimation.cu:339-429) is put
through the same synced step for comparison.
"""
from __future__ import annotations

import numpy as np


def rot_err_mrad(Ra, Rb) -> float:
    """Angle of Ra Rb^T in milliradians (atan2 of the skew part against the trace)."""
    R = np.asarray(Ra, np.float64) @ np.asarray(Rb, np.float64).T
    s = 0.5 * np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    return float(np.arctan2(np.linalg.norm(s), (np.trace(R) - 1.0) / 2.0) * 1000.0)


def pose_err(T, T64):
    """(translation error mm, rotation error mrad) of pose T against the FP64 pose."""
    T = np.asarray(T, np.float64)
    return float(np.linalg.norm(T[:3, 3] - T64[:3, 3])), rot_err_mrad(T[:3, :3], T64[:3, :3])


def synced_errors(oracle, h, seq, depths, modes=("icp", "frame"), with_float=True):
    """Per frame k = 1..n-1 and mode: the pose error of handle h's step from the FP64
    oracle's state after frame k-1.  Returns {mode: (n-1, 2) array of (mm, mrad)}, plus
    "float": the float oracle's ICP from the same pose and prediction."""
    from conftest import grid_spec

    gs = grid_spec(seq.cfg.grid)
    K = seq.K
    Ki = oracle.inv3(K)
    H, W = depths[0].shape
    p64 = oracle.pipeline64(H, W, gs, K)
    p64.initial(depths[0])
    out = {m: [] for m in modes}
    if with_float:
        out["float"] = []
    for k in range(1, len(depths)):
        T64p = p64.pose.copy()
        P64 = p64.prediction().astype(np.float32)
        vol = p64.volume() if "frame" in modes else None
        p64.incoming(depths[k])
        T64 = p64.pose.copy()
        Tp32 = T64p.astype(np.float32)
        for mode in modes:
            h.set_pose(Tp32)
            if mode == "icp":
                h.set_predicted(P64)
            else:
                h.set_volume(*vol)
                h.set_depth_u16(depths[k - 1])
                h.ray_casting()
            h.incoming_frame(depths[k])
            out[mode].append(pose_err(h.pose(), T64))
        if with_float:
            dk = oracle.depth_ingest(depths[k])
            v5, mask = oracle.vertex_normal(dk, Ki)
            cur6 = np.stack([v5[0], v5[1], dk, v5[2], v5[3], v5[4]])
            Tf, _ = oracle.estimate_pose(K, Tp32, cur6, mask, P64, iters=10)
            out["float"].append(pose_err(Tf, T64))
    p64.close()
    return {m: np.array(v) for m, v in out.items()}


def summary(err: np.ndarray) -> dict:
    """RMS and max of the per-frame translation (mm) and rotation (mrad) errors."""
    return {"frames": int(len(err)), "rms_mm": float(np.sqrt(np.mean(err[:, 0] ** 2))),
            "max_mm": float(err[:, 0].max()), "rms_mrad": float(np.sqrt(np.mean(err[:, 1] ** 2))),
            "max_mrad": float(err[:, 1].max())}
