"""Shared helpers for the test suite (comparison rules of the reference's unit tests)."""
from __future__ import annotations

import numpy as np


def ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    ia = np.asarray(a, dtype=np.float64).view(np.int64)
    ib = np.asarray(b, dtype=np.float64).view(np.int64)
    # map sign-magnitude to two's-complement ordering
    ia = np.where(ia < 0, np.int64(-0x8000000000000000) - ia, ia)
    ib = np.where(ib < 0, np.int64(-0x8000000000000000) - ib, ib)
    return np.abs(ia - ib)


def nearly_equal(fid, test, abs_eps: float = 1e-14, ulps: int = 4) -> np.ndarray:
    """testing_utilities::nearlyEqualDbl (src/utils/testing_utilities.h:85-86): equal when the
    absolute difference is <= 1e-14 or the two doubles are within 4 ULP."""
    fid = np.asarray(fid, dtype=np.float64)
    test = np.asarray(test, dtype=np.float64)
    return (np.abs(fid - test) <= abs_eps) | (ulp_diff(fid, test) <= ulps)


def real_slice(ng: int, one_d: bool = False):
    if one_d:
        return (slice(None), slice(ng, -ng))
    return (slice(None), slice(ng, -ng), slice(ng, -ng), slice(ng, -ng))
