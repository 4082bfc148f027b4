"""The C ABI library without a GPU: it loads, exports every symbol the public header
declares, carries the reference's defaults, and rejects invalid configurations before
touching the device."""
import ctypes as C
import subprocess

import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from kinect_fusion_slam_gb300 import _lib


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    declared = _lib.declared_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, missing
    # and the ctypes table covers exactly the header
    assert set(declared) == set(_lib.SIGNATURES)


def test_exported_symbols_via_nm():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    exported = {line.split()[-1] for line in out.stdout.splitlines() if " T kf_" in line}
    assert set(_lib.declared_symbols()) <= exported


def test_library_targets_sm103a_only():
    out = subprocess.run(["cuobjdump", "--list-elf", str(_lib.LIB_PATH)], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("cuobjdump unavailable")
    elves = [l for l in out.stdout.splitlines() if ".cubin" in l]
    assert elves and all("sm_103a" in l for l in elves)


def test_reference_defaults():
    c = _lib.default_config()
    assert (c.height, c.width) == (480, 640)  # system_interface.cpp:6-7
    assert (c.min_depth, c.max_depth) == (300.0, 2000.0)  # system_interface.cpp:10-11
    assert list(c.dims) == [360, 360, 300]  # kinfu_pipeline.h:46-48
    assert list(c.grid_start) == [-200, -200, -120]  # kinfu_pipeline.h:43-45
    assert c.voxel_size == 10.0
    assert (c.truncated_distance, c.sdf_minimum, c.sdf_maximum) == (300.0, -30.0, 300.0)
    assert c.icp_levels == 1 and c.icp_iterations[0] == 10  # sensor_pose_estimation.cu:339
    assert (c.icp_distance, c.icp_angle_deg) == (20.0, 30.0)  # :48, :69
    assert (c.bilateral, c.bilateral_radius, c.sigma_d, c.sigma_r) == (0, 3, 4.5, 30.0)
    assert c.tsdf_storage == kf.KF_TSDF_F32 and c.use_graphs == 1


@pytest.mark.parametrize("field,value", [
    ("height", 0), ("width", 1), ("dims", (2, 360, 300)), ("dims", (5000, 360, 300)),
    ("dims", (2048, 2048, 1024)), ("voxel_size", 0.0), ("truncated_distance", -1.0), ("icp_levels", 4),
    ("icp_levels", 0), ("icp_iterations", (65,)), ("tsdf_storage", 7), ("bilateral_radius", 8),
])
def test_invalid_config_rejected_without_device(field, value):
    lib = _lib.load()
    cfg = kf.make_config(**{field: value})
    h = _lib._H()
    assert lib.kf_create(C.byref(cfg), C.byref(h)) == _lib.KF_ERR_INVALID_ARGUMENT
    assert not h.value


def test_pyramid_config_limits():
    lib = _lib.load()
    h = _lib._H()
    # 3 levels need the size divisible by 4; 60 iterations per level exceed 64 per frame
    for kw in ({"icp_levels": 3, "height": 482}, {"icp_levels": 2, "icp_iterations": (40, 30)}):
        cfg = kf.make_config(**kw)
        assert lib.kf_create(C.byref(cfg), C.byref(h)) == _lib.KF_ERR_INVALID_ARGUMENT


def test_null_arguments():
    lib = _lib.load()
    assert lib.kf_create(None, None) == _lib.KF_ERR_INVALID_ARGUMENT
    assert lib.kf_destroy(None) == _lib.KF_ERR_INVALID_ARGUMENT
    assert lib.kf_last_error(None) == b"null handle"
    assert lib.kf_status_string(_lib.KF_ERR_CUDA) == b"CUDA error"


def test_load_depth_dat(tmp_path):
    raw = (np.arange(480 * 640) % 4000).astype(np.uint16).reshape(480, 640)
    raw.tofile(tmp_path / "dep0042.dat")
    assert np.array_equal(kf.load_depth_dat(tmp_path, 42), raw)
    with pytest.raises(kf.KinfuError):
        kf.load_depth_dat(tmp_path, 43)
    (tmp_path / "dep0044.dat").write_bytes(b"\0" * 100)  # truncated file
    with pytest.raises(kf.KinfuError):
        kf.load_depth_dat(tmp_path, 44)


def test_make_config_rejects_unknown_field():
    with pytest.raises(KeyError):
        kf.make_config(no_such_field=1)
