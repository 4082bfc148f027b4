"""kf_icp_associate_noalloc: the allocation-free ICP association + reduction.

Some callers cannot allocate device memory when they need this operator (a real-time
loop that must not stall on cudaMalloc, an application that owns all GPU memory
through its own pool).  The entry point takes caller-owned device buffers and keeps
its scratch in a static device array.  This test calls it through the C ABI, twice in
a row (the scratch keeps the previous call's contents, so the second call checks that
each call re-initialises what it must), and compares with the handle-based
kf_icp_associate: the same kernel in the same summation order, so the sums, count and
pairings must agree bit for bit.  This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import kinect_fusion_slam_gb300 as kf
from kinect_fusion_slam_gb300 import _lib
from conftest import grid_spec

pytestmark = pytest.mark.gpu


def _inputs(oracle, seq, depths):
    gs = grid_spec(seq.cfg.grid)
    K = seq.K
    Ki = oracle.inv3(K)
    t = np.full(gs.nvox, np.nan, np.float32)
    w = np.full(gs.nvox, np.nan, np.float32)
    T0 = seq.poses[0].astype(np.float32)
    d0 = oracle.depth_ingest(depths[0])
    oracle.integrate(gs, d0, K, Ki, T0, oracle.inv4(T0), t, w, first=True)
    pred6, _ = oracle.raycast(gs, d0, Ki, T0, t)
    d1 = oracle.depth_ingest(depths[1])
    return T0, d1, pred6


def test_noalloc_matches_handle_entry_point(oracle, small_seq):
    torch = pytest.importorskip("torch")  # only to own the caller's device buffers
    seq, depths = small_seq
    T0, d1, pred6 = _inputs(oracle, seq, depths)
    H, W = d1.shape
    h = kf.Handle(kf.make_config(height=H, width=W, dims=seq.cfg.grid.dims, grid_start=seq.cfg.grid.start,
                                 voxel_size=seq.cfg.grid.voxel_size))
    K = seq.K
    h.set_intrinsics(K[0, 0], K[1, 1], K[0, 2], K[1, 2])
    h.set_depth_f32(d1)
    v5, mask = h.calculate_vertices_and_normals()
    h.set_predicted(pred6)
    T = T0.copy()
    T[:3, 3] += np.float32(2.0)
    F = oracle.matmul4(oracle.inv4(T0), T)
    n_ref, sums_ref, pair_ref = h.icp_associate(F, T)
    assert n_ref > 200

    # the same maps the handle holds, in caller-owned device memory
    vmap = np.stack([v5[0], v5[1], d1, mask.astype(np.float32)], -1)
    nmap = np.stack([v5[2], v5[3], v5[4], np.zeros_like(d1)], -1)
    pv = np.stack([pred6[0], pred6[1], pred6[2], np.zeros_like(d1)], -1)
    pn = np.stack([pred6[3], pred6[4], pred6[5], np.zeros_like(d1)], -1)
    dev = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in (vmap, nmap, pv, pn)]
    lib = _lib.load()
    Kf = np.ascontiguousarray(K, np.float32).ravel()
    for call in range(2):
        sums = torch.full((28,), float("nan"), dtype=torch.float32, device="cuda")
        pair = torch.full((H * W,), -7, dtype=torch.int32, device="cuda")
        st = lib.kf_icp_associate_noalloc(H, W, Kf, F.ravel(), T.ravel(), *[C.c_void_p(t.data_ptr()) for t in dev],
                                          20.0, 30.0, C.c_void_p(sums.data_ptr()), C.c_void_p(pair.data_ptr()), None)
        torch.cuda.synchronize()
        assert st == _lib.KF_OK, f"call {call}: status {st}"
        s = sums.cpu().numpy()
        assert np.array_equal(s[:27].view(np.uint32), sums_ref.view(np.uint32)), f"call {call}: sums differ"
        assert int(s[27]) == n_ref
        assert np.array_equal(pair.cpu().numpy().reshape(H, W), pair_ref)


def test_noalloc_rejects_oversized_and_misaligned():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    eye = np.eye(4, dtype=np.float32).ravel()
    K = np.array([525, 0, 320.5, 0, 525, 240.5, 0, 0, 1], np.float32)
    buf = torch.zeros(4 * 700 * 500 + 4, dtype=torch.float32, device="cuda")
    out = torch.zeros(28, dtype=torch.float32, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    o = C.c_void_p(out.data_ptr())
    # beyond the static scratch's 640 x 480 limit
    assert lib.kf_icp_associate_noalloc(500, 700, K, eye, eye, p, p, p, p, 20.0, 30.0, o, None,
                                        None) == _lib.KF_ERR_UNSUPPORTED
    # float4 maps must be 16-byte aligned
    q = C.c_void_p(buf.data_ptr() + 4)
    assert lib.kf_icp_associate_noalloc(480, 640, K, eye, eye, q, p, p, p, 20.0, 30.0, o, None,
                                        None) == _lib.KF_ERR_INVALID_ARGUMENT
    assert lib.kf_icp_associate_noalloc(480, 640, K, eye, eye, p, p, p, p, 20.0, 30.0, None, None,
                                        None) == _lib.KF_ERR_INVALID_ARGUMENT
