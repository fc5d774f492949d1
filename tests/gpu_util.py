"""Helpers for the GPU parity tests."""
import numpy as np


def norm_rel_err(got, want):
    """max |got - want| / max |want| over a batch (per output column when 2-D)."""
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    if got.ndim == 1:
        den = np.max(np.abs(want))
        return float(np.max(np.abs(got - want)) / (den if den > 0 else 1.0))
    errs = []
    for k in range(want.shape[1]):
        den = np.max(np.abs(want[:, k]))
        errs.append(float(np.max(np.abs(got[:, k] - want[:, k])) / (den if den > 0 else 1.0)))
    return max(errs)
