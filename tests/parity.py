"""Shared comparison helpers of the parity tests."""
from __future__ import annotations

import numpy as np

# Per-sample radiance tolerance: 1e-4 relative (the project's parity bar for
# the float path), with an absolute floor for values near zero.
RTOL = 1e-4
ATOL = 1e-6
# Fraction of paths (pixels of a spp-1 frame) that must agree.
MIN_PATH_FRACTION = 0.999


def close_mask(a, b, rtol=RTOL, atol=ATOL):
    """Per pixel: every channel within atol + rtol * max(|a|, |b|)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    with np.errstate(invalid="ignore"):
        tol = atol + rtol * np.maximum(np.abs(a), np.abs(b))
        ok = (np.abs(a - b) <= tol) | (a == b)
    if ok.ndim == 3:
        ok = ok.all(axis=-1)
    return ok


def close_fraction(a, b, **kw):
    return float(close_mask(a, b, **kw).mean())


def tie_mask(hits_a_t, hits_b_t):
    """Prim-id disagreements that are exact ties in distance."""
    return np.asarray(hits_a_t).view(np.uint32) == np.asarray(hits_b_t).view(np.uint32)
