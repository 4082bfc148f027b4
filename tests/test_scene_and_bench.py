"""Host-side logic without a GPU: the synthetic sequence generator, the benchmark's
frame order, and the replicas' barrier / max-over-ranks on world_size 2 (gloo)."""
import os
import socket

import numpy as np
import pytest

from kinect_fusion_slam_gb300 import scene


def test_sequence_is_deterministic_and_seeded():
    a = scene.sequence(scene.config("c0"), frames=3)
    b = scene.sequence(scene.config("c0"), frames=3)
    c = scene.sequence(scene.config("c0", seed=99), frames=3)
    assert np.array_equal(a.depth(2), b.depth(2))
    assert np.array_equal(a.poses, b.poses)
    assert not np.array_equal(a.depth(2), c.depth(2))


def test_trajectory_statistics():
    s = scene.sequence(scene.config("c1"), frames=60)
    P = s.poses
    assert np.allclose(P[0], np.eye(4))
    steps = np.linalg.norm(np.diff(P[:, :3, 3], axis=0), axis=1)
    assert steps.min() >= 10.0 - 1e-9 and steps.max() <= 20.0 + 1e-9  # 1-2 cm per frame
    for k in range(1, 60):
        R = P[k - 1, :3, :3].T @ P[k, :3, :3]
        ang = np.degrees(np.arccos(np.clip((np.trace(R) - 1) / 2, -1, 1)))
        assert 0.49 <= ang <= 1.01  # 0.5-1 degree per frame
        assert np.allclose(P[k, :3, :3] @ P[k, :3, :3].T, np.eye(3), atol=1e-12)
    assert np.linalg.norm(P[:, :3, 3], axis=1).max() < 800.0  # stays near the room centre


def test_depth_noise_and_dropout():
    cfg = scene.config("c1")
    s = scene.sequence(cfg, frames=1)
    d = s.depth(0)
    assert d.dtype == np.uint16 and d.shape == (480, 640)
    zero = (d == 0).mean()
    assert 0.015 < zero < 0.03  # 2 % dropout
    clean = scene.render_depth_mm(scene.config("c1", noise=False, dropout=0.0), s.scene, s.poses[0], 0)
    m = (d > 0) & (clean > 0)
    err = d[m].astype(np.float64) - clean[m]
    z = clean[m] / 1000.0
    sigma_mm = 1000 * (0.0012 + 0.0019 * (z - 0.4) ** 2)
    assert abs(np.mean(err)) < 0.2
    assert 0.85 < np.std(err / sigma_mm) < 1.15


def test_intrinsics_reference_convention():
    K = scene.Camera().K_reference()
    assert K[0, 2] == 320.5 and K[1, 2] == 240.5  # 0-based 319.5 / 239.5 + 1
    small = scene.Camera().scaled(0.25)
    assert (small.width, small.height) == (160, 120)


def test_batch_configs_uneven():
    cfgs = scene.batch_configs()
    assert len(cfgs) == 16
    assert {c.grid.dims for c in cfgs} == {(128, 128, 128), (256, 256, 256), (384, 384, 320)}
    assert {(c.camera.width, c.camera.height) for c in cfgs} == {(640, 480), (320, 240)}


def test_pingpong_order():
    import bench

    o = bench.pingpong(4, 10)
    assert o == [0, 1, 2, 3, 2, 1, 0, 1, 2, 3]
    assert all(abs(a - b) == 1 for a, b in zip(o, o[1:]))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), KF_BENCH_BACKEND="gloo")
    import bench

    d = bench.Dist()
    d.barrier()
    out[rank] = d.max(10.0 + rank)
    d.barrier()
    d.close()


def test_replicas_max_over_ranks_gloo():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        procs = [mp.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        assert dict(out) == {0: 11.0, 1: 11.0}
