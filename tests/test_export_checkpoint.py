"""PLY export of the predicted surface (the viewer's point cloud, threeD_viewer.cpp:20-54)
and checkpoint save/load (resuming a run bit for bit)."""
import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from kinect_fusion_slam_gb300 import _lib

pytestmark = pytest.mark.gpu


def _handle(seq, H, W, **kw):
    g = seq.cfg.grid
    h = kf.Handle(kf.make_config(height=H, width=W, dims=g.dims, grid_start=g.start, voxel_size=g.voxel_size, **kw))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    return h


def _read_ply(path):
    data = open(path, "rb").read()
    end = data.index(b"end_header\n") + len(b"end_header\n")
    header = data[:end].decode()
    n = int([ln for ln in header.splitlines() if ln.startswith("element vertex")][0].split()[-1])
    rec = np.dtype([("p", "<f4", 3), ("n", "<f4", 3), ("rgb", "u1", 3)])
    body = np.frombuffer(data[end:], rec)
    assert body.size == n
    return header, body


def test_ply_export_matches_prediction(small_seq, tmp_path):
    seq, depths = small_seq
    H, W = depths.shape[1:]
    h = _handle(seq, H, W)
    h.initial_processing(depths[0])
    h.incoming_frame(depths[1])
    pred = h.predicted()
    keep = pred[2] != 0
    colour = (np.arange(H * W * 3) % 251).astype(np.uint8).reshape(H, W, 3)
    n = h.export_ply(tmp_path / "cloud.ply", colour)
    header, body = _read_ply(tmp_path / "cloud.ply")
    assert header.startswith("ply\nformat binary_little_endian 1.0\n")
    assert n == keep.sum() == body.size and n > 500
    # pixel order, world-space points and normals, the viewer's BGR -> RGB colour
    assert np.array_equal(body["p"], np.stack([pred[0][keep], pred[1][keep], pred[2][keep]], 1))
    assert np.array_equal(body["n"], np.stack([pred[3][keep], pred[4][keep], pred[5][keep]], 1))
    assert np.array_equal(body["rgb"], colour.reshape(-1, 3)[keep.ravel()][:, ::-1])
    # without a colour image the points are coloured by their normals
    assert h.export_ply(tmp_path / "plain.ply") == n


@pytest.mark.parametrize("storage", [kf.KF_TSDF_F32, kf.KF_TSDF_F16])
def test_checkpoint_resumes_bit_for_bit(small_seq, tmp_path, storage):
    seq, depths = small_seq
    H, W = depths.shape[1:]
    a = _handle(seq, H, W, tsdf_storage=storage)
    a.initial_processing(depths[0])
    a.incoming_frame(depths[1])
    a.save_checkpoint(tmp_path / "run.kfc")
    b = _handle(seq, H, W, tsdf_storage=storage)
    b.load_checkpoint(tmp_path / "run.kfc")
    assert np.array_equal(a.pose(), b.pose())
    for h in (a, b):
        h.incoming_frame(depths[2])
    assert np.array_equal(a.pose(), b.pose())
    ta, wa = a.volume()
    tb, wb = b.volume()
    assert np.array_equal(ta.view(np.uint32), tb.view(np.uint32))
    assert np.array_equal(wa.view(np.uint32), wb.view(np.uint32))
    assert np.array_equal(a.predicted().view(np.uint32), b.predicted().view(np.uint32))


def test_checkpoint_rejects_other_grid_and_foreign_files(small_seq, tmp_path):
    seq, depths = small_seq
    H, W = depths.shape[1:]
    a = _handle(seq, H, W)
    a.initial_processing(depths[0])
    a.save_checkpoint(tmp_path / "run.kfc")
    other = _handle(seq, H, W, tsdf_storage=kf.KF_TSDF_F16)
    with pytest.raises(kf.KinfuError) as e:
        other.load_checkpoint(tmp_path / "run.kfc")
    assert e.value.status == _lib.KF_ERR_INVALID_ARGUMENT
    (tmp_path / "junk.kfc").write_bytes(b"not a checkpoint" * 10)
    with pytest.raises(kf.KinfuError) as e:
        a.load_checkpoint(tmp_path / "junk.kfc")
    assert e.value.status == _lib.KF_ERR_IO
