"""Regenerate tests/golden/fp64_<workload>_traj.npz -- the FP64 oracle's trajectory on a
benchmark sequence.

Workload c1 (default): 640x480 depth into the 360x360x300 grid at 10 mm; workload c2:
the precision form's 512x512x430 grid at 7 mm.  Either way the first 48 frames of its
seeded synthetic sequence, i.e. the first forward pass of the benchmark's frame order.
Two trajectories are stored, both from the CPU oracles in oracle/:

  poses64  the FP64 oracle (kf_oracle64.cpp): the reference's algorithm in double
  poses32  the float oracle (kf_oracle.cpp): the reference's own float arithmetic,
           which the GPU's plain form reproduces bit for bit

The benchmark compares the GPU trajectories of both forms with poses64 (the absolute
trajectory error of the precision form), and poses32 against poses64 gives the
reference's own sensitivity to arithmetic precision on this sequence.

    python tests/golden/make_fp64_traj.py [c1|c2]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

FRAMES = 48


def main(workload: str = "c1") -> None:
    from kinect_fusion_slam_gb300 import scene
    from oracle.pyoracle import GridSpec, Oracle

    cfg = scene.config(workload)
    seq = scene.sequence(cfg, frames=FRAMES)
    depths = seq.depths(FRAMES)
    g = cfg.grid
    gs = GridSpec(tuple(g.dims), tuple(g.start), float(g.voxel_size), g.truncated_distance, g.sdf_minimum,
                  g.sdf_maximum)
    H, W = depths.shape[1:]
    o = Oracle()
    p64 = o.pipeline64(H, W, gs, seq.K)
    p32 = o.pipeline(H, W, gs, seq.K)
    poses64 = np.zeros((FRAMES, 4, 4))
    poses32 = np.zeros((FRAMES, 4, 4), np.float32)
    for k in range(FRAMES):
        for p in (p64, p32):
            (p.initial if k == 0 else p.incoming)(depths[k])
        poses64[k] = p64.pose
        poses32[k] = p32.pose
    p64.close()
    p32.close()
    np.savez_compressed(HERE / f"fp64_{workload}_traj.npz", poses64=poses64, poses32=poses32, frames=FRAMES,
                        workload=f"{workload} frames 0..47")
    err = np.linalg.norm(poses32[:, :3, 3] - poses64[:, :3, 3], axis=1)
    print(f"written; float oracle vs FP64 oracle: ATE {np.sqrt(np.mean(err ** 2)):.3f} mm, max {err.max():.3f} mm")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "c1")
