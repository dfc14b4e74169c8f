"""Shared comparison helpers for the parity tests."""
import numpy as np


def relerr(a, b):
    """max |a-b| scaled by the larger of max|b| and 1e-300."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    if a.size == 0:
        return 0.0
    scale = max(float(np.max(np.abs(b))), 1e-300)
    return float(np.max(np.abs(a - b))) / scale


def assert_close(a, b, tol, what=""):
    e = relerr(a, b)
    assert e <= tol, f"{what}: relative error {e:.3e} > {tol:.1e}"
