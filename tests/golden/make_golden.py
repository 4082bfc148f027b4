"""Regenerates tests/golden/*.npz from the reference's own kernel bodies.

Runs the reference (oracle/_ref: its CUDA kernel bodies compiled for the CPU by
oracle/build.py, which needs the reference tree) on small seeded synthetic
sequences and stores inputs and outputs compactly (sparse volumes, hit pixels only):

  pipeline_small.npz  160x120 depth, 180x180x150 grid @ 20 mm, initial + 3 frames:
                      per-frame poses, final volume, final prediction + hit voxels
  stages_small.npz    the same inputs through single stages: vertex/normal map, one
                      integration, one ray cast, one ICP association (sums), one
                      10-iteration pose estimate (per-iteration sums and poses)

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from kinect_fusion_slam_gb300 import scene  # noqa: E402
from oracle.pyoracle import GridSpec, Oracle, Reference  # noqa: E402


def small_sequence(frames=4, seed=21):
    cam = scene.Camera().scaled(0.25)
    g = scene.GridConfig((180, 180, 150), 20.0)
    cfg = scene.SceneConfig("golden", g, frames, camera=cam, seed=seed)
    seq = scene.sequence(cfg)
    return seq, seq.depths(frames), GridSpec(tuple(g.dims), tuple(g.start), g.voxel_size)


def sparse_volume(t, w):
    idx = np.flatnonzero(~np.isnan(w)).astype(np.int32)
    return idx, t[idx], w[idx]


def main():
    ref = Reference.load()
    if ref is None:
        raise SystemExit("reference kernels unavailable: the reference tree is needed to regenerate fixtures")
    o = Oracle()
    seq, depths, gs = small_sequence()
    H, W = depths.shape[1:]
    K = seq.K

    # ---- whole pipeline
    p = ref.pipeline(H, W, gs, K)
    p.initial(depths[0])
    poses = [p.pose]
    for k in range(1, len(depths)):
        p.incoming(depths[k])
        poses.append(p.pose)
    t, w = p.volume()
    vidx, vt, vw = sparse_volume(t, w)
    pred6, hit = p.prediction()
    hpx = np.flatnonzero(hit.ravel() >= 0).astype(np.int32)
    np.savez_compressed(HERE / "pipeline_small.npz", depths=depths, K=K, dims=np.array(gs.dims),
                        start=np.array(gs.start), voxel_size=np.float32(gs.voxel_size), poses=np.array(poses),
                        vol_idx=vidx, vol_tsdf=vt, vol_weight=vw, hit_px=hpx, hit_voxel=hit.ravel()[hpx],
                        pred=pred6.reshape(6, -1)[:, hpx])

    # ---- single stages
    Ki = o.inv3(K)
    d0, d1 = o.depth_ingest(depths[0]), o.depth_ingest(depths[1])
    v5, mask = ref.vertex_normal(d1, Ki)
    T0 = seq.poses[0].astype(np.float32)
    T1 = seq.poses[1].astype(np.float32)
    t = np.full(gs.nvox, np.nan, np.float32)
    w = np.full(gs.nvox, np.nan, np.float32)
    ref.integrate(gs, d0, K, Ki, T0, o.inv4(T0), t, w, first=True)
    ref.integrate(gs, d1, K, Ki, T1, o.inv4(T1), t, w, first=False)
    sidx, st, sw = sparse_volume(t, w)
    r6, rhit = ref.raycast(gs, d1, Ki, T1, t)
    rpx = np.flatnonzero(rhit.ravel() >= 0).astype(np.int32)
    cur6 = np.stack([v5[0], v5[1], d1, v5[2], v5[3], v5[4]])
    F = o.matmul4(o.inv4(T0), T1)
    _, sums42, flags = ref.icp_associate(K, F, T1, cur6, mask, r6)
    Te, log = ref.estimate_pose(K, T0, cur6, mask, r6, iters=10)
    np.savez_compressed(HERE / "stages_small.npz", depth0=d0, depth1=d1, K=K, Ki=Ki, T0=T0, T1=T1,
                        dims=np.array(gs.dims), start=np.array(gs.start), voxel_size=np.float32(gs.voxel_size),
                        vertex5=v5, mask=mask, vol_idx=sidx, vol_tsdf=st, vol_weight=sw, ray_px=rpx,
                        ray_voxel=rhit.ravel()[rpx], ray_pred=r6.reshape(6, -1)[:, rpx], icp_F=F, icp_sums42=sums42,
                        icp_flags=flags, pose_est=Te, pose_sums=log["sums"], pose_log=log["poses"])
    for f in ("pipeline_small.npz", "stages_small.npz"):
        print(f, (HERE / f).stat().st_size, "bytes")


if __name__ == "__main__":
    main()
