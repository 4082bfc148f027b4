"""The ICP pose update's float-float solve against its FP64 restatement, bit for bit.

cv::Cholesky and cv::Mat's product accumulate in double; the device computes those
results as float pairs with a proven error bound and decides each float by Ziv's test,
falling back to the FP64 sequence when undecided (csrc/kf_solve.cuh).  kf_selftest_solve
runs both on seeded random systems shaped like the ICP's normal equations (some of them
singular) and counts differences.
"""
import ctypes as C

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
