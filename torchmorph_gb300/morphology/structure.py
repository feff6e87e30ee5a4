"""Structuring-element helpers (host only), reference torchmorph/morphology/structure.py."""

from __future__ import annotations

import torch
from torch import Tensor


def _offset_grid(rank: int, radius: int, device=None) -> Tensor:
    axes = [torch.arange(-radius, radius + 1, device=device) for _ in range(rank)]
    return torch.stack(torch.meshgrid(*axes, indexing="ij"), dim=0)


def generate_binary_structure(rank: int, connectivity: int) -> Tensor:
    """Boolean 3^rank element whose entries lie within `connectivity` unit steps of the centre."""
    if connectivity < 1 or connectivity > rank:
        raise ValueError(f"connectivity must be in [1, rank], got {connectivity}")
    if rank < 1:
        raise ValueError(f"rank must be >= 1, got {rank}")
    return (_offset_grid(rank, 1) != 0).sum(dim=0) <= connectivity


def _generated_structure_connectivity(structure: Tensor) -> int | None:
    """The connectivity c if `structure` equals generate_binary_structure(ndim, c)."""
    if any(size != 3 for size in structure.shape):
        return None
    steps = (_offset_grid(structure.ndim, 1, structure.device) != 0).sum(dim=0)
    for c in range(1, structure.ndim + 1):
        if torch.equal(structure, steps <= c):
            return c
    return None


def _normalize_origin(origin: int | tuple[int, ...], ndim: int) -> tuple[int, ...]:
    if isinstance(origin, int):
        return (origin,) * ndim
    values = tuple(origin)
    if len(values) != ndim:
        raise ValueError(f"origin dimension is not {ndim}, got {len(values)}")
    return values


def _validate_origin(origin: tuple[int, ...], structure: Tensor, name: str = "origin") -> None:
    for o, size in zip(origin, structure.shape):
        if not -(size // 2) <= o <= (size - 1) // 2:
            raise ValueError(f"invalid {name}")


def iterate_structure(
    structure: Tensor,
    iterations: int,
    origin: int | tuple[int, ...] | None = None,
) -> Tensor | tuple[Tensor, list[int]]:
    """Dilate a binary structure with itself `iterations - 1` times."""
    structure = structure != 0
    if iterations < 2:
        result = structure.clone()
    else:
        conn = _generated_structure_connectivity(structure)
        out_shape = tuple(iterations * (s - 1) + 1 for s in structure.shape)
        if conn is not None:
            grid = _offset_grid(structure.ndim, iterations, structure.device)
            result = grid.abs().sum(dim=0) <= conn * iterations
        else:
            pts = torch.nonzero(structure, as_tuple=False)
            result = torch.zeros(out_shape, dtype=torch.bool, device=structure.device)
            if pts.numel() != 0:
                acc = pts
                for _ in range(iterations - 1):
                    acc = torch.unique((acc[:, None, :] + pts[None, :, :]).reshape(-1, structure.ndim),
                                       dim=0)
                result[tuple(acc.unbind(dim=1))] = True
    if origin is None:
        return result
    o = _normalize_origin(origin, structure.ndim)
    return result, [v * iterations for v in o]
