import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the CUDA library")
    config.addinivalue_line("markers", "slow: larger CPU cases")


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle

    return Oracle()


@pytest.fixture(scope="session")
def reference():
    """The reference's own kernel bodies compiled for the CPU (skips where the spliced
    sources are unavailable)."""
    from oracle.pyoracle import Reference

    r = Reference.load()
    if r is None:
        pytest.skip("reference kernels unavailable (no reference tree and no earlier splice)")
    return r


REAL_FRAMES = ROOT / "tests" / "golden" / "real_frames.npz"


def real_frame(i: int) -> np.ndarray:
    """The reference's recorded depth frame dep%04d.dat (640x480 uint16 mm): frames 25-27
    from the committed fixture (tests/golden/make_real_frames.py), others from the
    reference checkout named by KF_REF_DIR."""
    with np.load(REAL_FRAMES) as z:
        if f"dep{i:04d}" in z.files:
            return z[f"dep{i:04d}"].copy()
    ref = os.environ.get("KF_REF_DIR")
    if not ref:
        pytest.skip(f"dep{i:04d}.dat is not in the fixture and KF_REF_DIR is not set")
    return np.fromfile(Path(ref) / "data" / f"dep{i:04d}.dat", np.uint16).reshape(480, 640)


@pytest.fixture(scope="session")
def small_seq():
    """160x120 synthetic sequence on the c0 grid (180x180x150 at 20 mm; fast on CPU and GPU)."""
    from kinect_fusion_slam_gb300 import scene

    cam = scene.Camera().scaled(0.25)
    g = scene.GridConfig((180, 180, 150), 20.0)
    cfg = scene.SceneConfig("small", g, 4, camera=cam, seed=11)
    seq = scene.sequence(cfg)
    return seq, seq.depths(4)


@pytest.fixture(scope="session")
def c0_seq():
    """Config c0: 640x480, 180x180x150 grid at 20 mm, 20 frames."""
    from kinect_fusion_slam_gb300 import scene

    seq = scene.sequence("c0")
    return seq, seq.depths(seq.cfg.frames)


def grid_spec(g):
    from oracle.pyoracle import GridSpec

    return GridSpec(tuple(g.dims), tuple(g.start), float(g.voxel_size), g.truncated_distance, g.sdf_minimum,
                    g.sdf_maximum)
