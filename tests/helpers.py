"""Shared helpers for the parity tests."""
import numpy as np


def rel_inf(a, b):
    """max|a-b| / max|b| (norm-wise relative error)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    d = np.max(np.abs(a - b))
    s = np.max(np.abs(b))
    return float(d / s) if s > 0 else float(d)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
