"""The CPU oracle against golden vectors produced by the reference's own kernel bodies
(tests/golden/make_golden.py).  Bit-exact throughout; runs wherever the oracle
builds, including machines without the reference tree."""
from pathlib import Path

import numpy as np
import pytest

from oracle.pyoracle import GridSpec

GOLDEN = Path(__file__).resolve().parent / "golden"


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def stages():
    return dict(np.load(GOLDEN / "stages_small.npz"))


@pytest.fixture(scope="module")
def pipeline_fx():
    return dict(np.load(GOLDEN / "pipeline_small.npz"))


def spec(fx):
    return GridSpec(tuple(int(x) for x in fx["dims"]), tuple(int(x) for x in fx["start"]), float(fx["voxel_size"]))


def test_inverse_intrinsics(oracle, stages):
    assert np.array_equal(bits(oracle.inv3(stages["K"])), bits(stages["Ki"]))


def test_vertex_map(oracle, stages):
    v5, mask = oracle.vertex_normal(stages["depth1"], stages["Ki"])
    assert np.array_equal(mask, stages["mask"])
    assert np.array_equal(bits(v5), bits(stages["vertex5"]))


def test_integration(oracle, stages):
    gs = spec(stages)
    t = np.full(gs.nvox, np.nan, np.float32)
    w = np.full(gs.nvox, np.nan, np.float32)
    K, Ki, T0, T1 = stages["K"], stages["Ki"], stages["T0"], stages["T1"]
    oracle.integrate(gs, stages["depth0"], K, Ki, T0, oracle.inv4(T0), t, w, first=True)
    oracle.integrate(gs, stages["depth1"], K, Ki, T1, oracle.inv4(T1), t, w, first=False)
    idx = np.flatnonzero(~np.isnan(w))
    assert np.array_equal(idx, stages["vol_idx"])
    assert np.array_equal(bits(t[idx]), bits(stages["vol_tsdf"]))
    assert np.array_equal(bits(w[idx]), bits(stages["vol_weight"]))
    assert set(np.unique(w[idx])) <= {1.0, 2.0}


def _volume(stages):
    gs = spec(stages)
    t = np.full(gs.nvox, np.nan, np.float32)
    w = np.full(gs.nvox, np.nan, np.float32)
    t[stages["vol_idx"]] = stages["vol_tsdf"]
    w[stages["vol_idx"]] = stages["vol_weight"]
    return gs, t, w


def test_raycast(oracle, stages):
    gs, t, _ = _volume(stages)
    pred6, hit = oracle.raycast(gs, stages["depth1"], stages["Ki"], stages["T1"], t)
    px = np.flatnonzero(hit.ravel() >= 0)
    assert np.array_equal(px, stages["ray_px"])
    assert np.array_equal(hit.ravel()[px], stages["ray_voxel"])
    assert np.array_equal(bits(pred6.reshape(6, -1)[:, px]), bits(stages["ray_pred"]))


def _icp_inputs(oracle, stages):
    gs, t, _ = _volume(stages)
    pred6, _ = oracle.raycast(gs, stages["depth1"], stages["Ki"], stages["T1"], t)
    v5 = stages["vertex5"]
    cur6 = np.stack([v5[0], v5[1], stages["depth1"], v5[2], v5[3], v5[4]])
    return cur6, pred6


def test_icp_association(oracle, stages):
    cur6, pred6 = _icp_inputs(oracle, stages)
    n, sums, pair = oracle.icp_associate(stages["K"], stages["icp_F"], stages["T1"], cur6, stages["mask"], pred6)
    assert np.array_equal((pair >= 0).astype(np.int32), stages["icp_flags"])
    assert n == int(stages["icp_flags"].sum())
    assert np.array_equal(bits(sums), bits(stages["icp_sums42"]))


def test_estimate_pose(oracle, stages):
    cur6, pred6 = _icp_inputs(oracle, stages)
    T, log = oracle.estimate_pose(stages["K"], stages["T0"], cur6, stages["mask"], pred6, iters=10)
    assert np.array_equal(bits(log["sums"]), bits(stages["pose_sums"]))
    assert np.array_equal(bits(log["poses"]), bits(stages["pose_log"]))
    assert np.array_equal(bits(T), bits(stages["pose_est"]))


def test_pipeline(oracle, pipeline_fx):
    fx = pipeline_fx
    gs = spec(fx)
    depths = fx["depths"]
    H, W = depths.shape[1:]
    p = oracle.pipeline(H, W, gs, fx["K"])
    p.initial(depths[0])
    assert np.array_equal(bits(p.pose), bits(fx["poses"][0]))
    for k in range(1, len(depths)):
        p.incoming(depths[k])
        assert np.array_equal(bits(p.pose), bits(fx["poses"][k])), f"frame {k}"
    t, w = p.volume()
    idx = np.flatnonzero(~np.isnan(w))
    assert np.array_equal(idx, fx["vol_idx"])
    assert np.array_equal(bits(t[idx]), bits(fx["vol_tsdf"]))
    assert np.array_equal(bits(w[idx]), bits(fx["vol_weight"]))
    pred6, hit = p.prediction()
    px = np.flatnonzero(hit.ravel() >= 0)
    assert np.array_equal(px, fx["hit_px"])
    assert np.array_equal(hit.ravel()[px], fx["hit_voxel"])
    assert np.array_equal(bits(pred6.reshape(6, -1)[:, px]), bits(fx["pred"]))
