"""The C++ host side: include/kinfu_pipeline.hpp (the reference's KinfuPipeline /
SystemUtility interface over the C ABI) and the headless frame loop built on it
(kinect_fusion_slam_gb300/driver/kinfu_run.cpp, the reference's system_interface.cpp
without the viewer).

On the CPU: the header compiles on its own and kinfu_run is built and rejects bad
arguments.  On the GPU: kinfu_run, reading dep%04d.dat frames as the reference does,
produces the same poses, bit for bit, as the Python binding driving the same library
on the same frames, in both forms."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
DRIVER = ROOT / "kinect_fusion_slam_gb300" / "lib" / "kinfu_run"


def _built():
    from kinect_fusion_slam_gb300 import build

    build.build()
    return DRIVER


def test_header_compiles_alone(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "t.cpp"
    src.write_text('#include "kinfu_pipeline.hpp"\nint main() { Kinfu::Plane p(2, 3); return p.at(1, 2) != 0.f; }\n')
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), "-c", str(src),
                        "-o", str(tmp_path / "t.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_kinfu_run_rejects_bad_arguments():
    drv = _built()
    r = subprocess.run([str(drv), "--bogus"], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr
    r = subprocess.run([str(drv), "--start", "5", "--end", "4"], capture_output=True, text=True)
    assert r.returncode == 2


def _write_frames(d: Path, depths, first: int):
    for k, f in enumerate(depths):
        (d / f"dep{first + k:04d}.dat").write_bytes(np.ascontiguousarray(f, dtype="<u2").tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [False, True])
def test_kinfu_run_poses_match_python_binding(tmp_path, precision):
    import kinect_fusion_slam_gb300 as kf
    from kinect_fusion_slam_gb300 import scene

    drv = _built()
    seq = scene.sequence(scene.config("c1"), frames=5)
    depths = seq.depths(5)
    _write_frames(tmp_path, depths, 25)
    out = tmp_path / "poses.bin"
    args = [str(drv), "--data", str(tmp_path), "--start", "25", "--end", "29", "--poses", str(out), "--quiet"]
    if precision:
        args.append("--precision")
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "frames/s" in r.stdout
    poses = np.fromfile(out, np.float32).reshape(-1, 4, 4)
    assert poses.shape[0] == 5

    extra = dict(tsdf_storage=kf.KF_TSDF_F16, solve_mode=kf.KF_SOLVE_PRECISE,
                 icp_reduction=kf.KF_REDUCE_TREE) if precision else {}
    h = kf.Handle(kf.make_config(height=480, width=640, **extra))  # reference grid and intrinsics
    h.initial_processing(depths[0])
    ref = [h.pose()]
    for k in range(1, 5):
        h.incoming_frame(depths[k])
        ref.append(h.pose())
    h.close()
    assert np.array_equal(poses.view(np.uint32), np.array(ref, np.float32).view(np.uint32))
    assert np.abs(poses[-1, :3, 3] - poses[0, :3, 3]).max() > 1.0  # the camera moved and was tracked
