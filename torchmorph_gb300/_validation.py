"""Argument contract of the (B, C, *spatial) operators.

Same checks and messages as the reference's torchmorph/_validation.py:8-42.
"""

from __future__ import annotations

from collections.abc import Sequence

from torch import Tensor

MAX_SPATIAL_NDIM = 8


def validate_bcs_input(input: Tensor) -> int:
    """Check a (B, C, *spatial) CUDA tensor and return its number of spatial dims."""
    if not input.is_cuda:
        raise ValueError("Input tensor must be on CUDA device.")
    if input.ndim < 3:
        raise ValueError(
            f"Input must be (B, C, Spatial...) with at least 3 dimensions, got {input.shape}."
        )
    nd = input.ndim - 2
    if nd > MAX_SPATIAL_NDIM:
        raise ValueError(f"Input spatial dimensions must be in range 1 to 8, got {nd}.")
    if input.numel() == 0:
        raise ValueError(f"Invalid input: empty tensor with shape {input.shape}.")
    return nd


def validate_output(
    input: Tensor,
    output: Tensor | None,
    expected_shape: Sequence[int] | None = None,
    name: str = "output",
) -> None:
    """Check that an optional preallocated output has the expected shape and device."""
    if output is None:
        return
    want = tuple(input.shape) if expected_shape is None else tuple(expected_shape)
    if tuple(output.shape) != want:
        raise ValueError(f"{name} shape {tuple(output.shape)} must match expected shape {want}")
    if output.device != input.device:
        raise ValueError(
            f"{name} must be on the same device as input, got {output.device} and {input.device}"
        )
