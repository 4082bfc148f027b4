"""Writes tests/golden/real_frames.npz: three of the reference's recorded Kinect depth
frames (data/dep0025.dat - dep0027.dat, 640x480 uint16 millimetres, as
SystemUtility::LoadDepthData reads them at system_utility.cpp:58-68), so that the GPU
parity tests can run the CUDA path against the oracle on real sensor depth -- holes,
edges and noise that the synthetic room does not have -- on machines without the
reference tree.

The frames are part of PoChang007/Kinect_Fusion_SLAM, MIT License, Copyright (c) 2021
Po-Chang Su; the notice travels with them in tests/golden/REAL_FRAMES_NOTICE.txt.

Usage: KF_REF_DIR=<reference checkout> python tests/golden/make_real_frames.py
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
FRAMES = (25, 26, 27)
H, W = 480, 640


def main() -> int:
    ref = os.environ.get("KF_REF_DIR")
    if not ref:
        print("set KF_REF_DIR to the reference checkout", file=sys.stderr)
        return 2
    data = Path(ref) / "data"
    arrs = {}
    for i in FRAMES:
        raw = np.fromfile(data / f"dep{i:04d}.dat", np.uint16)
        if raw.size != H * W:
            print(f"dep{i:04d}.dat: {raw.size} values, expected {H * W}", file=sys.stderr)
            return 1
        arrs[f"dep{i:04d}"] = raw.reshape(H, W)
    np.savez_compressed(HERE / "real_frames.npz", frames=np.array(FRAMES, np.int32), **arrs)
    print(f"wrote {HERE / 'real_frames.npz'}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
