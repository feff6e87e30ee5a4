"""Ragged batches of 2-D images or 3-D volumes: one persistent launch per operator.

A :class:`RaggedBatch` packs items of different sizes -- all 2-D images or
all 3-D volumes -- one after another in a single flat CUDA buffer and keeps
a device plan with one descriptor per item.  Every operator here runs as ONE
launch over the tiles of all items (libtmcore ``tm_ragged_*`` for images,
``tm_ragged3d_*`` for volumes, ``tm_ragged_edt`` for the distance transform)
instead of one launch per item; the result for each item is bit-identical to
the uniform-batch operator applied to ``item[None, None]`` (``grey_erosion``
... in ``torchmorph_gb300.morphology`` and
``euclidean_distance_transform``, i.e. the reference's
``torchmorph/morphology/grey.py``, ``binary.py`` and
``distance_transform.py:72-102``).

The plan depends only on the image shapes, so batches derived from one
another share it, and a fixed sequence of operators can be captured once into
a CUDA graph and replayed (:func:`capture`).  Operators on batches sharing a
plan must not run concurrently on different streams (the plan holds the
tile queue of the running launch).
"""

from __future__ import annotations

from typing import Callable, Sequence

import torch
from torch import Tensor

from . import _lib
from .morphology.grey import _MODE_MAP, _resolve_element
from .morphology.structure import _normalize_origin, _validate_origin, generate_binary_structure

_TM_ERR_UNSUPPORTED = 2  # tm_status of a call outside a kernel's limits


class RaggedBatch:
    """Items of different shapes (all 2-D or all 3-D) packed in one contiguous 1-D CUDA buffer."""

    def __init__(self, data: Tensor, shapes: Sequence[Sequence[int]], offsets: Sequence[int] | None = None,
                 plan: Tensor | None = None):
        if data.dim() != 1 or not data.is_contiguous():
            raise ValueError("RaggedBatch data must be a contiguous 1-D tensor")
        self.data = data
        self.shapes = [tuple(int(v) for v in sh) for sh in shapes]
        if not self.shapes:
            raise ValueError("a RaggedBatch needs at least one image")
        nd = len(self.shapes[0])
        if nd not in (2, 3) or any(len(sh) != nd for sh in self.shapes):
            raise ValueError("RaggedBatch items must all be 2-D or all be 3-D")
        if any(v < 1 for sh in self.shapes for v in sh):
            raise ValueError("RaggedBatch images must be non-empty")
        sizes = [_numel(sh) for sh in self.shapes]
        if offsets is None:
            offsets, pos = [], 0
            for n in sizes:
                offsets.append(pos)
                pos += n
        self.offsets = [int(o) for o in offsets]
        end = max(o + n for o, n in zip(self.offsets, sizes))
        if min(self.offsets) < 0 or end > data.numel():
            raise ValueError("RaggedBatch offsets run outside the data buffer")
        self._plan = plan
        self._edt_plan = None

    @classmethod
    def from_images(cls, images: Sequence[Tensor]) -> "RaggedBatch":
        """Pack items of shape (H, W) or (D, H, W) (or with leading (1, 1)) into one buffer (a copy)."""
        if len(images) == 0:
            raise ValueError("a RaggedBatch needs at least one image")
        flat, shapes = [], []
        for im in images:
            if im.dim() in (4, 5) and im.shape[0] == 1 and im.shape[1] == 1:
                im = im[0, 0]
            if im.dim() not in (2, 3):
                raise ValueError("RaggedBatch images must be (H, W) or (1, 1, H, W), volumes (D, H, W) "
                                 "or (1, 1, D, H, W)")
            shapes.append(tuple(im.shape))
            flat.append(im.reshape(-1))
        return cls(torch.cat(flat).contiguous(), shapes)

    def __len__(self) -> int:
        return len(self.shapes)

    def __getitem__(self, i: int) -> Tensor:
        o = self.offsets[i]
        return self.data[o:o + _numel(self.shapes[i])].view(self.shapes[i])

    def images(self) -> list[Tensor]:
        return [self[i] for i in range(len(self))]

    @property
    def ndim(self) -> int:
        """Spatial dimensions of the items (2 or 3)."""
        return len(self.shapes[0])

    @property
    def device(self):
        return self.data.device

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def numel(self) -> int:
        return sum(_numel(sh) for sh in self.shapes)

    @property
    def plan(self) -> Tensor:
        """Device descriptor table (built on first use, shared with derived batches)."""
        if self._plan is None:
            if not self.data.is_cuda:
                raise ValueError("ragged operators need a CUDA RaggedBatch")
            lib = _lib.load()
            n = len(self.shapes)
            dims = list(zip(*self.shapes))
            with torch.cuda.device(self.data.device):
                if self.ndim == 2:
                    nbytes = lib.tm_ragged_plan_size(n)
                    plan = torch.empty(int(nbytes), dtype=torch.uint8, device=self.data.device)
                    _lib.check(lib.tm_ragged_plan(n, _lib.i64_array(dims[0]), _lib.i64_array(dims[1]),
                                                  _lib.i64_array(self.offsets), _lib.ptr(plan), nbytes,
                                                  _lib.stream_of(self.data.device)), "tm_ragged_plan")
                else:
                    nbytes = lib.tm_ragged3d_plan_size(n)
                    plan = torch.empty(int(nbytes), dtype=torch.uint8, device=self.data.device)
                    _lib.check(lib.tm_ragged3d_plan(n, _lib.i64_array(dims[0]), _lib.i64_array(dims[1]),
                                                    _lib.i64_array(dims[2]), _lib.i64_array(self.offsets),
                                                    _lib.ptr(plan), nbytes, _lib.stream_of(self.data.device)),
                               "tm_ragged3d_plan")
            self._plan = plan
        return self._plan

    def with_data(self, data: Tensor) -> "RaggedBatch":
        """A batch with the same layout (and plan) over another buffer."""
        if data.shape != self.data.shape:
            raise ValueError("data must have the layout's buffer size")
        return RaggedBatch(data, self.shapes, self.offsets, self._plan)

    def empty_like(self, dtype=None) -> "RaggedBatch":
        return self.with_data(torch.empty_like(self.data, dtype=dtype or self.data.dtype))

    def map(self, fn: Callable[[Tensor], Tensor]) -> "RaggedBatch":
        """Elementwise op on the whole buffer in one launch (e.g. ``lambda x: x > 0.5``)."""
        return self.with_data(fn(self.data).contiguous())


def _numel(shape) -> int:
    n = 1
    for v in shape:
        n *= int(v)
    return n


def _check_batch(batch: RaggedBatch, dtype, what: str):
    if not isinstance(batch, RaggedBatch):
        raise TypeError(f"{what} expects a RaggedBatch")
    if not batch.data.is_cuda:
        raise ValueError("Input tensor must be on CUDA device.")
    if batch.dtype != dtype:
        raise ValueError(f"{what} needs a {dtype} RaggedBatch, got {batch.dtype}")


def _output(batch: RaggedBatch, output: RaggedBatch | None, dtype) -> RaggedBatch:
    if output is None:
        return batch.empty_like(dtype)
    if output.shapes != batch.shapes or output.offsets != batch.offsets or output.dtype != dtype:
        raise ValueError("output must be a RaggedBatch with the input's layout and dtype")
    if output.data.data_ptr() == batch.data.data_ptr():
        raise ValueError("output must not alias the input")
    if output._plan is None:
        output._plan = batch._plan
    return output


def _grey(name, batch, size, footprint, structure, mode, cval, origin, output):
    _check_batch(batch, torch.float32, name)
    nd = batch.ndim
    if nd == 3:
        name = name.replace("tm_ragged_", "tm_ragged3d_")
    struct, fp = _resolve_element(nd, size, footprint, structure)
    o = _normalize_origin(origin, nd)
    _validate_origin(o, struct)
    if mode not in _MODE_MAP:
        raise ValueError(f"Unknown mode '{mode}'. Must be one of {list(_MODE_MAP.keys())}.")
    plan = batch.plan  # built before the output so that the output shares it
    out = _output(batch, output, torch.float32)
    lib = _lib.load()
    fp_ptr = None if fp.numel() == 0 else _lib.ctypes_u8(fp)
    with torch.cuda.device(batch.device):
        _lib.check(getattr(lib, name)(_lib.ptr(batch.data), _lib.ptr(out.data), _lib.ptr(plan), plan.numel(),
                                      len(batch), _lib.ctypes_f32(struct), fp_ptr,
                                      _lib.i64_array(struct.shape), _lib.i64_array(o), _MODE_MAP[mode],
                                      float(cval), _lib.stream_of(batch.device)), name)
    return out


def grey_erosion(batch: RaggedBatch, size=None, footprint=None, structure=None, mode="reflect", cval=0.0,
                 origin=0, output: RaggedBatch | None = None) -> RaggedBatch:
    """Per-item grey erosion of a float32 RaggedBatch, one launch for all items."""
    return _grey("tm_ragged_grey_erosion", batch, size, footprint, structure, mode, cval, origin, output)


def grey_dilation(batch: RaggedBatch, size=None, footprint=None, structure=None, mode="reflect", cval=0.0,
                  origin=0, output: RaggedBatch | None = None) -> RaggedBatch:
    """Per-item grey dilation of a float32 RaggedBatch, one launch for all items."""
    return _grey("tm_ragged_grey_dilation", batch, size, footprint, structure, mode, cval, origin, output)


def grey_opening(batch, size=None, footprint=None, structure=None, mode="reflect", cval=0.0, origin=0):
    tmp = grey_erosion(batch, size, footprint, structure, mode, cval, origin)
    return grey_dilation(tmp, size, footprint, structure, mode, cval, origin)


def grey_closing(batch, size=None, footprint=None, structure=None, mode="reflect", cval=0.0, origin=0):
    tmp = grey_dilation(batch, size, footprint, structure, mode, cval, origin)
    return grey_erosion(tmp, size, footprint, structure, mode, cval, origin)


def _binary(name, batch, structure, border_value, origin, output):
    _check_batch(batch, torch.bool, name)
    nd = batch.ndim
    if nd == 3:
        name = name.replace("tm_ragged_", "tm_ragged3d_")
    if structure is None:
        structure = generate_binary_structure(nd, 1)
    if structure.ndim != nd:
        raise ValueError(f"structure dimension is not {nd}, got {structure.ndim}")
    st = (structure != 0).detach().to(device="cpu", dtype=torch.bool).contiguous()
    o = _normalize_origin(origin, nd)
    _validate_origin(o, st)
    plan = batch.plan
    out = _output(batch, output, torch.bool)
    if not bool(st.any()):  # the reference's empty-structure result
        out.data.fill_(name.endswith("erosion"))
        return out
    lib = _lib.load()
    with torch.cuda.device(batch.device):
        _lib.check(getattr(lib, name)(_lib.ptr(batch.data), _lib.ptr(out.data), _lib.ptr(plan), plan.numel(),
                                      len(batch), _lib.ctypes_u8(st), _lib.i64_array(st.shape),
                                      _lib.i64_array(o), int(bool(border_value)),
                                      _lib.stream_of(batch.device)), name)
    return out


def binary_erosion(batch: RaggedBatch, structure=None, border_value=False, origin=0,
                   output: RaggedBatch | None = None) -> RaggedBatch:
    """Per-item binary erosion (one iteration, no mask) of a bool RaggedBatch."""
    return _binary("tm_ragged_binary_erosion", batch, structure, border_value, origin, output)


def binary_dilation(batch: RaggedBatch, structure=None, border_value=False, origin=0,
                    output: RaggedBatch | None = None) -> RaggedBatch:
    """Per-item binary dilation (one iteration, no mask) of a bool RaggedBatch."""
    return _binary("tm_ragged_binary_dilation", batch, structure, border_value, origin, output)


def binary_opening(batch, structure=None, border_value=False, origin=0):
    """Per-item binary opening; 2-D items in one pass on bit-packed tiles."""
    if batch.ndim == 2:
        try:
            return _binary("tm_ragged_binary_opening", batch, structure, border_value, origin, None)
        except _lib.TorchmorphError as e:
            if e.status != _TM_ERR_UNSUPPORTED:
                raise
    return binary_dilation(binary_erosion(batch, structure, border_value, origin), structure, border_value,
                           origin)


def binary_closing(batch, structure=None, border_value=False, origin=0):
    """Per-item binary closing; 2-D items in one pass on bit-packed tiles."""
    if batch.ndim == 2:
        try:
            return _binary("tm_ragged_binary_closing", batch, structure, border_value, origin, None)
        except _lib.TorchmorphError as e:
            if e.status != _TM_ERR_UNSUPPORTED:
                raise
    return binary_erosion(binary_dilation(batch, structure, border_value, origin), structure, border_value,
                          origin)


def euclidean_distance_transform(batch: RaggedBatch, return_distances: bool = True,
                                 return_indices: bool = False):
    """Exact Euclidean distance transform (unit sampling) of every item of a ragged batch
    of 2-D images or 3-D volumes, in ONE launch for all items (libtmcore
    ``tm_ragged_edt``).  Item by item the result equals
    ``euclidean_distance_transform(item[None, None])`` (reference
    ``distance_transform.py:72-102``): the distance to the nearest background (zero)
    voxel, ties to the smallest last-axis coordinate as scipy.ndimage breaks them, and
    the virtual site (-1, 0, ...) for an item without background.

    Returns the distances as a float32 RaggedBatch with the input's layout, and/or the
    feature indices as an int32 tensor (ndim, batch.data.numel()) whose plane d holds,
    at every packed voxel, coordinate d of its nearest background voxel inside its item.
    """
    if not isinstance(batch, RaggedBatch):
        raise TypeError("euclidean_distance_transform expects a RaggedBatch")
    if not batch.data.is_cuda:
        raise ValueError("Input tensor must be on CUDA device.")
    if not return_distances and not return_indices:
        raise ValueError("At least one of return_distances or return_indices must be True.")
    if batch.dtype in (torch.bool, torch.uint8):
        data, in_dtype = batch.data.view(torch.uint8), _lib.TM_U8
    elif batch.dtype == torch.float32:
        data, in_dtype = batch.data, _lib.TM_F32
    else:
        raise ValueError(f"ragged EDT needs a bool, uint8 or float32 RaggedBatch, got {batch.dtype}")
    lib = _lib.load()
    n, nd, total = len(batch), batch.ndim, batch.data.numel()
    dev = batch.device
    with torch.cuda.device(dev):
        stream = _lib.stream_of(dev)
        plan = batch._edt_plan
        if plan is None:
            nbytes = lib.tm_ragged_edt_plan_size(n)
            plan = torch.empty(int(nbytes), dtype=torch.uint8, device=dev)
            flat_shapes = [v for sh in batch.shapes for v in sh]
            _lib.check(lib.tm_ragged_edt_plan(n, nd, _lib.i64_array(flat_shapes), _lib.i64_array(batch.offsets),
                                              _lib.ptr(plan), nbytes, stream), "tm_ragged_edt_plan")
            batch._edt_plan = plan
        lines = [sum(_numel(sh) // sh[a] for sh in batch.shapes) for a in range(nd)]
        max_line = max(max(sh) for sh in batch.shapes)
        wbytes = lib.tm_ragged_edt_workspace_size(total, max_line)
        ws = torch.empty(int(wbytes), dtype=torch.uint8, device=dev)
        dist = torch.empty(total, dtype=torch.float32, device=dev) if return_distances else None
        idx = torch.empty((nd, total), dtype=torch.int32, device=dev) if return_indices else None
        _lib.check(lib.tm_ragged_edt(_lib.ptr(data), in_dtype, _lib.ptr(plan), plan.numel(), n, nd, total, max_line,
                                     _lib.i64_array(lines), _lib.ptr(dist), _lib.ptr(idx), None, _lib.ptr(ws), wbytes,
                                     stream), "tm_ragged_edt")
    out = []
    if return_distances:
        out.append(RaggedBatch(dist, batch.shapes, batch.offsets, batch._plan))
    if return_indices:
        out.append(idx)
    return out[0] if len(out) == 1 else tuple(out)


def capture(fn: Callable, *args, warmup: int = 1):
    """Capture fn(*args) into a CUDA graph; returns (graph, outputs of the captured call).

    ``graph.replay()`` reruns every launch of fn on the same buffers; the
    outputs are the graph's own buffers, overwritten by each replay.
    """
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(warmup):
            fn(*args)
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        out = fn(*args)
    return graph, out
