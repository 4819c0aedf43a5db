"""Shared numeric helpers for the test suite."""
import numpy as np


def bits(a):
    """float64 array -> int64 bit patterns (so -0.0 != 0.0)."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64)).view(np.int64)


def assert_bits_equal(actual, expected, what=""):
    a, e = bits(actual), bits(expected)
    if a.shape != e.shape or not np.array_equal(a, e):
        bad = np.flatnonzero(a.ravel() != e.ravel())[:8]
        raise AssertionError(
            f"{what}: not bit-identical at flat indices {bad.tolist()}: "
            f"{np.asarray(actual).ravel()[bad].tolist()} vs {np.asarray(expected).ravel()[bad].tolist()}")


def ulp_diff(a, b):
    """Distance in units in the last place between two float64 arrays."""
    ia = bits(a).astype(np.int64)
    ib = bits(b).astype(np.int64)
    ia = np.where(ia < 0, np.int64(-(2**63)) - ia, ia)
    ib = np.where(ib < 0, np.int64(-(2**63)) - ib, ib)
    return np.abs(ia - ib)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d
