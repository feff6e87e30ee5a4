"""Distance-transform front end (reference torchmorph/distance_transform.py).

Same signatures, return conventions and error messages as the reference.
Differences that only remove work: boolean / uint8 / float32 inputs go to
the kernels without a float32 copy, and preallocated float32 / int32 outputs
are written in place instead of through a temporary.
"""

from __future__ import annotations

import math
from collections.abc import Sequence

import torch
from torch import Tensor

from . import _C
from ._validation import validate_bcs_input, validate_output


def _normalize_sampling(sampling, spatial_ndim: int) -> list[float]:
    if sampling is None:
        values = [1.0] * spatial_ndim
    elif isinstance(sampling, (int, float)):
        values = [float(sampling)] * spatial_ndim
    else:
        values = [float(v) for v in sampling]
        if len(values) == 1:
            values *= spatial_ndim
        elif len(values) != spatial_ndim:
            raise ValueError(f"sampling must have length 1 or {spatial_ndim}, got {len(values)}")
    if any(not math.isfinite(v) or v <= 0 for v in values):
        raise ValueError("sampling values must be finite and greater than zero")
    return values


def _prepare_distance_transform(input, return_distances, return_indices, distances, indices):
    nd = validate_bcs_input(input)
    validate_output(input, distances, name="distances")
    validate_output(input, indices, (nd, *input.shape), name="indices")
    return_distances = return_distances or distances is not None
    return_indices = return_indices or indices is not None
    if not return_distances and not return_indices:
        raise ValueError("At least one distance transform output must be requested.")
    return nd, return_distances, return_indices


def _kernel_input(input: Tensor) -> Tensor:
    """Foreground carrier for the kernels: nonzero means foreground, as float32 in the reference."""
    x = input.detach()
    if x.dtype in (torch.float32, torch.bool):
        return x.contiguous()
    if x.dtype == torch.uint8:
        return (x != 0).contiguous()
    return x.float().contiguous()


def _direct(out: Tensor | None, dtype) -> Tensor | None:
    """`out` itself when the kernel can write it in place."""
    if out is not None and out.dtype == dtype and out.is_contiguous():
        return out
    return None


def _finish(raw_d, raw_i, return_distances, return_indices, distances, indices):
    if distances is not None and raw_d is not None and raw_d is not distances:
        distances.copy_(raw_d)
    if indices is not None and raw_i is not None and raw_i is not indices:
        indices.copy_(raw_i)
    ret_d = return_distances and distances is None
    ret_i = return_indices and indices is None
    if ret_d and ret_i:
        return raw_d, raw_i
    if ret_d:
        return raw_d
    if ret_i:
        return raw_i
    return None


def euclidean_distance_transform(
    input: Tensor,
    sampling: float | Sequence[float] | None = None,
    return_distances: bool = True,
    return_indices: bool = False,
    distances: Tensor | None = None,
    indices: Tensor | None = None,
):
    """Exact Euclidean distance transform of a (B, C, *spatial) CUDA tensor."""
    nd, rd, ri = _prepare_distance_transform(input, return_distances, return_indices, distances,
                                             indices)
    samp = _normalize_sampling(sampling, nd)
    raw_d, raw_i, _ = _C.edt(_kernel_input(input), samp, rd, ri,
                             distances_out=_direct(distances, torch.float32),
                             indices_out=_direct(indices, torch.int32))
    return _finish(raw_d, raw_i, rd, ri, distances, indices)


def euclidean_distance_transform_squared(input: Tensor) -> Tensor:
    """Exact int32 squared Euclidean distances (unit spacing) -- not in the reference."""
    validate_bcs_input(input)
    _, _, sq = _C.edt(_kernel_input(input), None, False, False, sqdist=True)
    return sq


_CDT_ALIASES = {"cityblock": "taxicab", "manhattan": "taxicab"}


def chamfer_distance_transform(
    input: Tensor,
    metric: str = "chessboard",
    return_distances: bool = True,
    return_indices: bool = False,
    distances: Tensor | None = None,
    indices: Tensor | None = None,
):
    """Chamfer distance transform of a (B, C, *spatial) CUDA tensor.

    metric: 'chessboard', 'taxicab' (aliases 'cityblock', 'manhattan'), or
    'chamfer345' (weighted 3-4-5 chamfer divided by 3, 1-3 spatial dims).
    """
    _, rd, ri = _prepare_distance_transform(input, return_distances, return_indices, distances,
                                            indices)
    metric = _CDT_ALIASES.get(metric, metric)
    if metric not in {"chessboard", "taxicab", "chamfer345"}:
        raise ValueError(
            "metric must be 'chessboard', 'taxicab', 'cityblock', 'manhattan' or 'chamfer345'."
        )
    raw_d, raw_i = _C.cdt(_kernel_input(input), metric, rd, ri,
                          distances_out=_direct(distances, torch.float32),
                          indices_out=_direct(indices, torch.int32))
    return _finish(raw_d, raw_i, rd, ri, distances, indices)


def brute_force_distance_transform(
    input: Tensor,
    metric: str = "euclidean",
    sampling: float | Sequence[float] | None = None,
    return_distances: bool = True,
    return_indices: bool = False,
    distances: Tensor | None = None,
    indices: Tensor | None = None,
):
    """Brute-force distance transform of a (B, C, *spatial) CUDA tensor."""
    nd, rd, ri = _prepare_distance_transform(input, return_distances, return_indices, distances,
                                             indices)
    if metric not in {"euclidean", "taxicab", "chessboard"}:
        raise ValueError("metric must be 'euclidean', 'taxicab', or 'chessboard'.")
    samp = _normalize_sampling(sampling, nd)
    raw_d, raw_i = _C.bfdt(_kernel_input(input), metric, samp, rd, ri,
                           distances_out=_direct(distances, torch.float32),
                           indices_out=_direct(indices, torch.int32))
    return _finish(raw_d, raw_i, rd, ri, distances, indices)
