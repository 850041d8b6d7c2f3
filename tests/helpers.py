"""Shared helpers of the test suite."""
import numpy as np


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def per_field_rel(a, b):
    """Relative L2 error of each velocity component (u, v, w)."""
    return [rel_l2(a[c], b[c]) for c in range(a.shape[0])]
