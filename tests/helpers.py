"""Shared helpers of the parity tests (per-item scipy application, seeded inputs)."""

import numpy as np


def per_item(x, fn, **kw):
    """Apply fn to every (b, c) item of a (B, C, *S) array; fn returns one array."""
    x = np.asarray(x)
    s = x.shape[2:]
    out = [np.asarray(fn(t, **kw)) for t in x.reshape(-1, *s)]
    return np.stack(out).reshape(x.shape[:2] + out[0].shape)


def per_item_indices(x, fn, **kw):
    """Per-item (distances, indices) with indices laid out (ndim, B, C, *S)."""
    x = np.asarray(x)
    s = x.shape[2:]
    res = [fn(t, return_indices=True, **kw) for t in x.reshape(-1, *s)]
    d = np.stack([r[0] for r in res]).reshape(x.shape)
    i = np.stack([r[1] for r in res], axis=1).reshape((len(s),) + x.shape)
    return d, i


def rng(seed=0):
    return np.random.default_rng(seed)
