"""The ray walk's per-position tests, restated in Python over every class of float value
(positive, +0, -0, negative, NaN, infinities, subnormals).

1. The kernel's branch-free form (`trace` in csrc/kf_tsdf.cu) decides each position as
   the reference's loop does (voxel_traversal.cu:207-222: stop at NaN after a negative
   value, a negative value after NaN, or a positive value after a negative one; the zero
   crossing is the first negative value right after a positive one).
2. The fast path's condition -- the previous value is not negative and no value of the
   group is negative -- implies that every position of the group advances.
3. The fast path's integer keys (`negative_key`) are below their limit exactly for the
   values that compare < 0, in FP32 and in FP16 storage.
"""
import itertools
import math

import numpy as np

VALUES = [1.0, 0.5, 1e-40, 0.0, -0.0, -1e-40, -0.5, -1.0, math.inf, -math.inf, math.nan]


def reference_step(prev, cur):
    """'stop', 'cross' or 'advance' for one position of the reference's loop."""
    if math.isnan(cur) and prev < 0:
        return "stop"
    if cur < 0 and math.isnan(prev):
        return "stop"
    if cur > 0 and prev < 0:
        return "stop"
    if cur < 0 and prev > 0:
        return "cross"
    return "advance"


def kernel_step(prev, cur):
    """The kernel's form for a live position (inside the bounds, walk not ended)."""
    stop = (not (cur <= 0.0)) if prev < 0.0 else (math.isnan(prev) and cur < 0.0)
    cross = (not stop) and prev > 0.0 and cur < 0.0
    adv = (not stop) and (not cross)
    return "stop" if stop else "cross" if cross else "advance" if adv else "?"


def test_kernel_step_is_the_reference_step():
    for prev, cur in itertools.product(VALUES + [0.0], VALUES):
        assert kernel_step(prev, cur) == reference_step(prev, cur), (prev, cur)


def test_fast_group_condition_implies_every_position_advances():
    not_negative = [v for v in VALUES if not v < 0]
    for prev in [v for v in VALUES if not v < 0]:
        for group in itertools.product(not_negative, repeat=4):
            p = prev
            for cur in group:
                assert kernel_step(p, cur) == "advance", (prev, group)
                p = cur


def test_negative_keys():
    # FP32: bits - 0x80000001 < 0x7f800000 exactly for values < 0
    rng = np.random.default_rng(7)
    bits = np.concatenate([rng.integers(0, 1 << 32, 1 << 20, dtype=np.uint64).astype(np.uint32),
                           np.array([0, 1, 0x7f800000, 0x7f800001, 0x7fffffff, 0x80000000, 0x80000001,
                                     0xff7fffff, 0xff800000, 0xff800001, 0xffffffff], np.uint32)])
    with np.errstate(invalid="ignore"):
        neg = bits.view(np.float32) < 0
    key = (bits.astype(np.uint64) - 0x80000001) % (1 << 32)
    assert np.array_equal(key < 0x7f800000, neg)
    # FP16 (value in the low half of the stored pair): (pair << 16) - 0x80010000 < 0x7c000000
    h = np.arange(1 << 16, dtype=np.uint64)
    pair = h | (rng.integers(0, 1 << 16, h.size, dtype=np.uint64) << np.uint64(16))
    with np.errstate(invalid="ignore"):
        neg16 = h.astype(np.uint16).view(np.float16) < 0
    key16 = ((pair << np.uint64(16)) - np.uint64(0x80010000)) % (1 << 32)
    assert np.array_equal(key16 < 0x7c000000, neg16)
