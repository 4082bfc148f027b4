"""The ICP pose update's float-float solve against its FP64 restatement, bit for bit.

cv::Cholesky and cv::Mat's product accumulate in double; the device computes those
results as float pairs with a proven error bound and decides each float by Ziv's test,
falling back to the FP64 sequence when undecided (csrc/kf_solve.cuh).  kf_selftest_solve
runs both on seeded random systems shaped like the ICP's normal equations (some of them
singular) and counts differences.
"""
import ctypes as C

import numpy as np
import pytest

from kinect_fusion_slam_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("seed", [1, 2024])
def test_float_float_solve_is_bit_identical(seed):
    lib = _lib.load()
    counts = (C.c_ulonglong * 5)()
    assert lib.kf_selftest_solve(seed, 152 * 2, 64, counts) == _lib.KF_OK
    systems, solve_diff, outcome_diff, not_pd, product_diff = list(counts)
    assert systems == 152 * 2 * 4 * 64
    assert not_pd > 0.05 * systems  # the mix includes rank-deficient systems
    assert solve_diff == 0
    assert outcome_diff == 0
    assert product_diff == 0


def test_selftest_rejects_bad_arguments():
    lib = _lib.load()
    counts = (C.c_ulonglong * 5)()
    assert lib.kf_selftest_solve(1, 0, 64, counts) == _lib.KF_ERR_INVALID_ARGUMENT
    assert lib.kf_selftest_solve(1, 4, 64, None) == _lib.KF_ERR_INVALID_ARGUMENT


def _icp_like_systems(rng, n):
    """Sums of rows a = (v x m, m) with v up to a few metres (mm) and unit m over 3 to
    400 rows -- the shape of the ICP's normal equations; the short ones are singular."""
    A = np.zeros((n, 6, 6))
    b = np.zeros((n, 6))
    for k in range(n):
        rows = int(rng.choice([3, 5, 6, 8, 64, 400]))
        scale = 1.0 + 3000.0 * rng.random()
        v = scale * np.column_stack([rng.uniform(-1, 1, rows), rng.uniform(-1, 1, rows),
                                     rng.uniform(1.0, 2.0, rows)])
        m = rng.normal(size=(rows, 3))
        m /= np.linalg.norm(m, axis=1, keepdims=True)
        a = np.hstack([np.cross(v, m), m])
        r = 20.0 * rng.uniform(-1, 1, rows)
        A[k] = a.T @ a
        b[k] = a.T @ r
    return A, b


def test_fp64_solve_against_numpy():
    """The precision form's FP64 solve (fraction-free Gauss-Jordan by a warp pair, one
    series-refined reciprocal per row) against numpy's FP64 solve: the same
    positive-definite decision away from the boundary, and solutions within 1e-12
    relative (scaled by the system's condition number) where it solves."""
    rng = np.random.default_rng(7)
    n = 4096
    A, b = _icp_like_systems(rng, n)
    x = np.zeros((n, 6))
    ok = np.zeros(n, np.int32)
    lib = _lib.load()
    st = lib.kf_selftest_solve6(A.ctypes.data, b.ctypes.data, x.ctypes.data, ok.ctypes.data, n)
    assert st == _lib.KF_OK
    n_pd = 0
    for k in range(n):
        w = np.linalg.eigvalsh(A[k])
        ratio = w[0] / w[-1]
        if abs(ratio) < 1e-13:
            continue  # at the positive-definite boundary either decision is rounding
        pd = ratio > 0
        assert bool(ok[k]) == pd, (k, ratio)
        if pd:
            n_pd += 1
            xr = np.linalg.solve(A[k], b[k])
            err = np.linalg.norm(x[k] - xr) / max(np.linalg.norm(xr), 1e-300)
            assert err <= 1e-12 / ratio + 1e-14, (k, err, ratio)
    assert n_pd > 0.5 * n
    assert (ok == 0).sum() > 0.05 * n


def test_fp64_solve_far_from_unit_scale():
    """Systems scaled by powers of two (exact, the solution unchanged).  Near 2^-1010 and
    2^1012 the final divisions leave the refined reciprocal's range and fall back to
    IEEE division; with subnormal entries (2^-1060) the pivots are subnormal and the
    whole system is solved again by the IEEE Gauss-Jordan fallback.  The systems are
    well-conditioned and positive definite, so all three must match numpy's solve of the
    same system at unit scale."""
    rng = np.random.default_rng(11)
    n = 96
    A = np.zeros((n, 6, 6))
    for k in range(n):
        q = rng.normal(size=(6, 6))
        A[k] = q @ q.T + 6.0 * np.eye(6)
    b = rng.normal(size=(n, 6))
    ref = np.linalg.solve(A, b[..., None])[..., 0]
    scales = np.array([2.0 ** -1010, 2.0 ** -1060, 2.0 ** 1012])
    for sc in scales:
        As = A * sc
        bs = b * sc
        tiny = sc < 2.0 ** -1022
        if tiny:
            # the subnormal inputs are rounded: the reference is the rounded system
            ref_k = np.linalg.solve(As / sc, (bs / sc)[..., None])[..., 0]
        else:
            ref_k = ref
        x = np.zeros((n, 6))
        ok = np.zeros(n, np.int32)
        lib = _lib.load()
        st = lib.kf_selftest_solve6(As.ctypes.data, bs.ctypes.data, x.ctypes.data, ok.ctypes.data, n)
        assert st == _lib.KF_OK
        assert ok.all(), sc
        err = np.abs(x - ref_k).max() / np.abs(ref_k).max()
        # subnormal arithmetic keeps only an absolute 2^-1074 (~2^-17 of these entries)
        assert err <= (1e-3 if tiny else 1e-12), (sc, err)
