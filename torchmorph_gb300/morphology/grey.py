"""Grey morphology front end (reference torchmorph/morphology/grey.py).

Argument resolution, validation and error messages follow the reference
operator for operator; the arithmetic runs in libtmcore through ``_C``.
"""

from __future__ import annotations

import torch
from torch import Tensor

from .. import _C
from .._validation import validate_bcs_input, validate_output
from .structure import _normalize_origin, _validate_origin

_MODE_MAP = {
    "constant": 0,
    "reflect": 1,
    "nearest": 2,
    "mirror": 3,
    "wrap": 4,
}


def _element_kwargs(size, footprint, structure, mode, cval, origin) -> dict:
    return dict(size=size, footprint=footprint, structure=structure, mode=mode, cval=cval,
                origin=origin)


def _resolve_element(spatial_ndim, size, footprint, structure):
    """(structure float32 CPU, footprint bool CPU or empty) with priority structure > footprint > size."""
    fp_cpu = torch.empty(0, dtype=torch.bool)
    if structure is not None:
        struct = structure.to(torch.float32)
        if footprint is not None:
            mask = footprint.to(torch.bool)
            if tuple(mask.shape) != tuple(struct.shape):
                raise ValueError(
                    f"Footprint shape {tuple(mask.shape)} must match structure "
                    f"shape {tuple(struct.shape)}."
                )
            if not mask.any():
                raise ValueError("All-zero footprint is not supported.")
            fp_cpu = mask.detach().to(device="cpu", dtype=torch.bool).contiguous()
    elif footprint is not None:
        mask = footprint.to(torch.bool)
        if not mask.any():
            raise ValueError("All-zero footprint is not supported.")
        struct = torch.zeros(tuple(mask.shape), dtype=torch.float32)
        fp_cpu = mask.detach().to(device="cpu", dtype=torch.bool).contiguous()
    elif size is not None:
        if isinstance(size, int):
            size = (size,) * spatial_ndim
        if any(v <= 0 for v in size):
            raise ValueError("size values must be greater than zero")
        struct = torch.zeros(tuple(size), dtype=torch.float32)
    else:
        raise ValueError("At least one of size, footprint, or structure must be specified.")
    if struct.ndim != spatial_ndim:
        raise ValueError(
            f"Structure dimension {struct.ndim} must match spatial dimension {spatial_ndim}."
        )
    return struct.detach().to(device="cpu", dtype=torch.float32).contiguous(), fp_cpu


def _prepare(input, size, footprint, structure, mode, origin):
    nd = validate_bcs_input(input)
    struct, fp = _resolve_element(nd, size, footprint, structure)
    o = _normalize_origin(origin, nd)
    _validate_origin(o, struct)
    if mode not in _MODE_MAP:
        raise ValueError(f"Unknown mode '{mode}'. Must be one of {list(_MODE_MAP.keys())}.")
    return struct, fp, list(o), _MODE_MAP[mode]


def _grey_morphology(
    input: Tensor,
    size=None,
    footprint=None,
    structure=None,
    output=None,
    mode: str = "reflect",
    cval: float = 0.0,
    origin=0,
    *,
    operation: str,
    differentiable: bool = False,
) -> Tensor:
    validate_bcs_input(input)
    validate_output(input, output)
    struct, fp, o, m = _prepare(input, size, footprint, structure, mode, origin)
    if differentiable and input.requires_grad and torch.is_grad_enabled():
        result = _GreyMorphologyFunction.apply(input, struct, fp, o, m, cval, operation == "dilation")
        if output is not None:
            raise ValueError("output= is not supported for a differentiable call")
        return result
    kernel = _C.grey_erosion_cuda if operation == "erosion" else _C.grey_dilation_cuda
    result = kernel(input.detach().contiguous().float(), struct, fp, o, m, cval)
    if output is not None:
        output.copy_(result)
        return output
    return result


class _GreyMorphologyFunction(torch.autograd.Function):
    """Grey erosion/dilation with a hand-written backward: the forward records, per
    output, the first footprint tap attaining the extremum; the backward gathers each
    input's gradient from the outputs whose recorded tap reads it."""

    @staticmethod
    def forward(ctx, input, struct, fp, origin, mode, cval, dilation):
        kernel = _C.grey_dilation_arg if dilation else _C.grey_erosion_arg
        out, arg = kernel(input.detach().contiguous().float(), struct, fp, origin, mode, cval)
        ctx.save_for_backward(arg)
        ctx.meta = (list(struct.shape), fp, origin, mode, dilation, input.dtype)
        return out

    @staticmethod
    def backward(ctx, grad_output):
        (arg,) = ctx.saved_tensors
        sshape, fp, origin, mode, dilation, dtype = ctx.meta
        grad = _C.grey_morphology_backward(grad_output, arg, sshape, fp, origin, mode, dilation)
        return grad.to(dtype), None, None, None, None, None, None


def grey_erosion(input, size=None, footprint=None, structure=None, output=None, mode="reflect",
                 cval=0.0, origin=0, *, differentiable=False) -> Tensor:
    """N-dimensional grey erosion of a (B, C, *spatial) CUDA tensor, computed in float32.

    ``differentiable=True`` (opt-in; 1-3 spatial dims, <= 255 footprint taps) makes the
    result track gradients w.r.t. ``input`` when it requires grad: the gradient of each
    output goes to the input voxel its first minimising tap read."""
    return _grey_morphology(input, size, footprint, structure, output, mode, cval, origin,
                            operation="erosion", differentiable=differentiable)


def grey_dilation(input, size=None, footprint=None, structure=None, output=None, mode="reflect",
                  cval=0.0, origin=0, *, differentiable=False) -> Tensor:
    """N-dimensional grey dilation of a (B, C, *spatial) CUDA tensor, computed in float32.

    ``differentiable=True``: see :func:`grey_erosion` (first maximising tap)."""
    return _grey_morphology(input, size, footprint, structure, output, mode, cval, origin,
                            operation="dilation", differentiable=differentiable)


def _fused(kind, input, output, differentiable, size, footprint, structure, mode, cval, origin):
    """The one-pass composite of 1-D / 2-D items with flat boxes (None elsewhere, and
    for differentiable calls, which compose the operators)."""
    validate_bcs_input(input)
    validate_output(input, output)
    if differentiable and input.requires_grad and torch.is_grad_enabled():
        return None
    return _one_pass(kind, input, size, footprint, structure, mode, cval, origin)


def grey_opening(input, size=None, footprint=None, structure=None, output=None, mode="reflect",
                 cval=0.0, origin=0, *, differentiable=False) -> Tensor:
    """Grey opening: dilation of the erosion (1-D / 2-D flat boxes: one pass)."""
    res = _fused("opening", input, output, differentiable, size, footprint, structure, mode, cval, origin)
    if res is not None:
        return _finish(res, output)
    kw = _element_kwargs(size, footprint, structure, mode, cval, origin)
    return grey_dilation(grey_erosion(input, differentiable=differentiable, **kw), output=output,
                         differentiable=differentiable, **kw)


def grey_closing(input, size=None, footprint=None, structure=None, output=None, mode="reflect",
                 cval=0.0, origin=0, *, differentiable=False) -> Tensor:
    """Grey closing: erosion of the dilation (1-D / 2-D flat boxes: one pass)."""
    res = _fused("closing", input, output, differentiable, size, footprint, structure, mode, cval, origin)
    if res is not None:
        return _finish(res, output)
    kw = _element_kwargs(size, footprint, structure, mode, cval, origin)
    return grey_erosion(grey_dilation(input, differentiable=differentiable, **kw), output=output,
                        differentiable=differentiable, **kw)


def _finish(result, output):
    if output is not None:
        output.copy_(result)
        return output
    return result


def _one_pass(kind, input, size, footprint, structure, mode, cval, origin):
    """The one-pass 2-D composite kernel's result, or None outside its limits."""
    struct, fp, o, m = _prepare(input, size, footprint, structure, mode, origin)
    return _C.grey_composite(kind, input.detach().contiguous().float(), struct, fp, o, m, cval)


def morphological_gradient(input, size=None, footprint=None, structure=None, output=None,
                           mode="reflect", cval=0.0, origin=0, *, differentiable=False) -> Tensor:
    """Dilation minus erosion (2-D items with elements of up to 64 taps: one pass)."""
    validate_bcs_input(input)
    validate_output(input, output)
    if not (differentiable and input.requires_grad and torch.is_grad_enabled()):
        res = _one_pass("gradient", input, size, footprint, structure, mode, cval, origin)
        if res is not None:
            return _finish(res, output)
    kw = _element_kwargs(size, footprint, structure, mode, cval, origin)
    return _finish(grey_dilation(input, differentiable=differentiable, **kw)
                   - grey_erosion(input, differentiable=differentiable, **kw), output)


def white_tophat(input, size=None, footprint=None, structure=None, output=None, mode="reflect",
                 cval=0.0, origin=0) -> Tensor:
    """Input minus its grey opening (1-D / 2-D flat boxes: one pass)."""
    res = _fused("white_tophat", input, output, False, size, footprint, structure, mode, cval, origin)
    if res is not None:
        return _finish(res, output)
    opened = grey_opening(input, **_element_kwargs(size, footprint, structure, mode, cval, origin))
    return _finish(input.detach().float() - opened, output)


def black_tophat(input, size=None, footprint=None, structure=None, output=None, mode="reflect",
                 cval=0.0, origin=0) -> Tensor:
    """Grey closing minus the input (1-D / 2-D flat boxes: one pass)."""
    res = _fused("black_tophat", input, output, False, size, footprint, structure, mode, cval, origin)
    if res is not None:
        return _finish(res, output)
    closed = grey_closing(input, **_element_kwargs(size, footprint, structure, mode, cval, origin))
    return _finish(closed - input.detach().float(), output)


def morphological_laplace(input, size=None, footprint=None, structure=None, output=None,
                          mode="reflect", cval=0.0, origin=0) -> Tensor:
    """Dilation plus erosion minus twice the input (2-D items with elements of up to 64 taps:
    one pass)."""
    validate_bcs_input(input)
    validate_output(input, output)
    res = _one_pass("laplace", input, size, footprint, structure, mode, cval, origin)
    if res is not None:
        return _finish(res, output)
    kw = _element_kwargs(size, footprint, structure, mode, cval, origin)
    res = grey_dilation(input, **kw) + grey_erosion(input, **kw) - 2 * input.detach().float()
    return _finish(res, output)
