"""Shared helpers of the parity tests (per-item scipy application, seeded inputs)."""

import numpy as np
import torch


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


def torch_grey_fp64(x, structure, footprint=None, origin=None, mode="reflect", cval=0.0,
                    dilation=False):
    """Grey erosion/dilation of a float64 (B, C, *S) torch tensor built from gathers and a
    min/max over the stacked taps, so torch autograd gives the FP64 reference gradient
    (torch.max/min over a dimension routes to the first extremum, the same tie rule)."""
    import oracle

    shape = tuple(x.shape[2:])
    n = int(np.prod(shape))
    flat = torch.cat([x.reshape(x.shape[0], x.shape[1], n),
                      torch.full((x.shape[0], x.shape[1], 1), float(cval), dtype=x.dtype)], -1)
    grids = np.meshgrid(*[np.arange(s) for s in shape], indexing="ij")
    vals = []
    for off, val in oracle._grey_taps(structure, footprint, origin, dilation):
        idx = [oracle.map_coords(g + o, s, mode) for g, o, s in zip(grids, off, shape)]
        valid = np.logical_and.reduce([i >= 0 for i in idx])
        lin = np.ravel_multi_index(tuple(np.where(valid, i, 0) for i in idx), shape)
        lin = torch.from_numpy(np.where(valid, lin, n).reshape(-1))
        v = flat[:, :, lin].reshape(x.shape)
        vals.append(v + float(val) if dilation else v - float(val))
    st = torch.stack(vals, 0)
    return st.max(0).values if dilation else st.min(0).values
