"""Binary morphology front end (reference torchmorph/morphology/binary.py).

Argument handling and error messages follow the reference; each erosion or
dilation step is one libtmcore launch through ``_C``.
"""

from __future__ import annotations

import functools

import torch
from torch import Tensor

from .. import _C
from .._validation import validate_bcs_input, validate_output
from .structure import _normalize_origin, _validate_origin, generate_binary_structure


@functools.lru_cache(maxsize=None)
def _default_structure(nd: int) -> Tensor:
    """The default element (cross, connectivity 1), built once per rank; read only."""
    return generate_binary_structure(nd, 1)


def _normalize_structure(structure: Tensor, spatial_ndim: int, name: str = "structure") -> Tensor:
    if structure.ndim != spatial_ndim:
        raise ValueError(f"{name} dimension is not {spatial_ndim}, got {structure.ndim}")
    return (structure != 0).detach().to(device="cpu", dtype=torch.bool).contiguous()


def _binary_morphology_cuda_step(input, structure, border_value, origin, *, mode):
    """One erosion/dilation launch; `structure` is a CPU bool tensor."""
    x = input if input.dtype == torch.bool and input.is_contiguous() else (input != 0).contiguous()
    kernel = _C.binary_erosion_cuda if mode == "erosion" else _C.binary_dilation_cuda
    return kernel(x, structure, list(origin), bool(border_value))


def _binary_morphology(input, structure, iterations, mask, output, border_value, origin, *, mode):
    until_stable = iterations < 1
    nd = validate_bcs_input(input)
    validate_output(input, output)
    if structure is None:
        structure = _default_structure(nd)
    structure = _normalize_structure(structure, nd)
    origin = _normalize_origin(origin, nd)
    _validate_origin(origin, structure)
    # foreground as bool (a bool input is used as is: comparing it with 0 is a slow
    # promoted elementwise pass)
    x = input.contiguous() if input.dtype == torch.bool else input != 0
    original = x
    if mask is not None and mask.shape != input.shape:
        raise ValueError(f"mask shape {mask.shape} must match input shape {input.shape}")
    mask_b = mask.to(device=input.device, dtype=torch.bool) if mask is not None else None
    empty = not bool(structure.any())  # CPU tensor: no device sync

    def step(v):
        if empty:
            return torch.full_like(v, mode == "erosion", dtype=torch.bool)
        return _binary_morphology_cuda_step(v, structure, border_value, origin, mode=mode)

    if until_stable:
        # Iterate to the fixed point without a host sync per iteration: run
        # chunks of 1, 2, 4, ... 32 iterations, each recording on the device
        # whether it changed anything, and read the flags once per chunk.
        # Once an iteration changes nothing every later one returns the same
        # volume, so a chunk with an unchanged iteration ends at the fixed
        # point (at most 31 iterations beyond it are computed).
        chunk = 1
        while True:
            changed = torch.empty(chunk, dtype=torch.bool, device=x.device)
            for j in range(chunk):
                nxt = step(x)
                if mask_b is not None:
                    nxt = torch.where(mask_b, nxt, original)
                changed[j] = torch.ne(nxt, x).any()
                x = nxt
            if not bool(changed.all()):
                break
            chunk = min(2 * chunk, 32)
    else:
        for _ in range(iterations):
            x = step(x)
            if mask_b is not None:
                x = torch.where(mask_b, x, original)
    result = x.to(dtype=torch.bool)
    if output is not None:
        output.copy_(result)
        return output
    return result


def binary_erosion(input, structure=None, iterations=1, mask=None, output=None, border_value=False,
                   origin=0) -> Tensor:
    """N-dimensional binary erosion of a (B, C, *spatial) CUDA tensor."""
    return _binary_morphology(input, structure, iterations, mask, output, border_value, origin,
                              mode="erosion")


def binary_dilation(input, structure=None, iterations=1, mask=None, output=None, border_value=False,
                    origin=0) -> Tensor:
    """N-dimensional binary dilation of a (B, C, *spatial) CUDA tensor."""
    return _binary_morphology(input, structure, iterations, mask, output, border_value, origin,
                              mode="dilation")


def binary_propagation(input, structure=None, mask=None, output=None, border_value=False,
                       origin=0) -> Tensor:
    """Dilation repeated until stable inside `mask`."""
    return _binary_morphology(input, structure, -1, mask, output, border_value, origin,
                              mode="dilation")


def binary_fill_holes(input, structure=None, output=None, origin=0) -> Tensor:
    """Fill the background regions not connected to the border."""
    validate_bcs_input(input)
    validate_output(input, output)
    outside = binary_propagation(torch.zeros_like(input, dtype=torch.bool), structure=structure,
                                 mask=torch.logical_not(input) if input.dtype == torch.bool else input == 0,
                                 output=None, border_value=True, origin=origin)
    result = torch.logical_not(outside)
    if output is not None:
        output.copy_(result)
        return output
    return result


def binary_hit_or_miss(input, structure1=None, structure2=None, output=None, origin1=0,
                       origin2=None) -> Tensor:
    """Voxels where structure1 fits the foreground and structure2 fits the background."""
    nd = validate_bcs_input(input)
    validate_output(input, output)
    origin1 = _normalize_origin(origin1, nd)
    origin2 = origin1 if origin2 is None else _normalize_origin(origin2, nd)
    if structure1 is None:
        structure1 = generate_binary_structure(nd, 1)
    structure1 = _normalize_structure(structure1, nd, "structure1")
    _validate_origin(origin1, structure1, "origin1")
    if structure2 is None:
        structure2 = torch.logical_not(structure1).contiguous()
    else:
        structure2 = _normalize_structure(structure2, nd, "structure2")
    _validate_origin(origin2, structure2, "origin2")
    fg = input if input.dtype == torch.bool else input != 0
    if bool(structure1.any()):
        hit = binary_erosion(fg, structure=structure1, origin=origin1)
    else:
        hit = torch.ones_like(fg, dtype=torch.bool)
    if bool(structure2.any()):
        result = torch.logical_and(hit, binary_erosion(torch.logical_not(fg), structure=structure2, origin=origin2))
    else:
        result = hit
    if output is not None:
        output.copy_(result)
        return output
    return result


def _one_pass(kind, input, structure, iterations, mask, output, border_value, origin):
    """The one-pass opening / closing of 1-D / 2-D items (one iteration, no mask) on
    bit-packed tiles; None where the reference's composition of two operators runs."""
    if iterations != 1 or mask is not None:
        return None
    nd = validate_bcs_input(input)
    validate_output(input, output)
    if nd > 2:
        return None
    if structure is None:
        structure = _default_structure(nd)
    structure = _normalize_structure(structure, nd)
    origin = _normalize_origin(origin, nd)
    _validate_origin(origin, structure)
    if not bool(structure.any()):
        return None
    x = input if input.dtype == torch.bool and input.is_contiguous() else (input != 0).contiguous()
    res = _C.binary_composite(kind, x, structure, list(origin), bool(border_value))
    if res is None:
        return None
    if output is not None:
        output.copy_(res)
        return output
    return res


def binary_opening(input, structure=None, iterations=1, mask=None, output=None, border_value=False,
                   origin=0) -> Tensor:
    """Erosion followed by dilation (1-D / 2-D, one iteration: one pass)."""
    res = _one_pass("opening", input, structure, iterations, mask, output, border_value, origin)
    if res is not None:
        return res
    x = binary_erosion(input, structure, iterations, mask, None, border_value, origin)
    return binary_dilation(x, structure, iterations, mask, output, border_value, origin)


def binary_closing(input, structure=None, iterations=1, mask=None, output=None, border_value=False,
                   origin=0) -> Tensor:
    """Dilation followed by erosion (1-D / 2-D, one iteration: one pass)."""
    res = _one_pass("closing", input, structure, iterations, mask, output, border_value, origin)
    if res is not None:
        return res
    x = binary_dilation(input, structure, iterations, mask, None, border_value, origin)
    return binary_erosion(x, structure, iterations, mask, output, border_value, origin)
