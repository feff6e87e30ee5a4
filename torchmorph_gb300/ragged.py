"""Ragged batches of 2-D images: one persistent launch per operator.

A :class:`RaggedBatch` packs 2-D images of different sizes one after another
in a single flat CUDA buffer and keeps a device plan with one descriptor per
image.  Every operator here runs as ONE launch over the tiles of all images
(libtmcore ``tm_ragged_*``) instead of one launch per image; the result for
each image is bit-identical to the uniform-batch operator applied to
``image[None, None]`` (``grey_erosion`` ... in ``torchmorph_gb300.morphology``,
i.e. the reference's ``torchmorph/morphology/grey.py`` and ``binary.py``).

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


class RaggedBatch:
    """2-D images of different shapes packed in one contiguous 1-D CUDA buffer."""

    def __init__(self, data: Tensor, shapes: Sequence[Sequence[int]], offsets: Sequence[int] | None = None,
                 plan: Tensor | None = None):
        if data.dim() != 1 or not data.is_contiguous():
            raise ValueError("RaggedBatch data must be a contiguous 1-D tensor")
        self.data = data
        self.shapes = [(int(h), int(w)) for h, w in shapes]
        if not self.shapes:
            raise ValueError("a RaggedBatch needs at least one image")
        if any(h < 1 or w < 1 for h, w in self.shapes):
            raise ValueError("RaggedBatch images must be non-empty")
        if offsets is None:
            offsets, pos = [], 0
            for h, w in self.shapes:
                offsets.append(pos)
                pos += h * w
        self.offsets = [int(o) for o in offsets]
        end = max(o + h * w for o, (h, w) in zip(self.offsets, self.shapes))
        if min(self.offsets) < 0 or end > data.numel():
            raise ValueError("RaggedBatch offsets run outside the data buffer")
        self._plan = plan

    @classmethod
    def from_images(cls, images: Sequence[Tensor]) -> "RaggedBatch":
        """Pack images of shape (H, W) (or (1, 1, H, W)) into one buffer (a copy)."""
        if len(images) == 0:
            raise ValueError("a RaggedBatch needs at least one image")
        flat, shapes = [], []
        for im in images:
            if im.dim() == 4 and im.shape[0] == 1 and im.shape[1] == 1:
                im = im[0, 0]
            if im.dim() != 2:
                raise ValueError("RaggedBatch images must be (H, W) or (1, 1, H, W)")
            shapes.append(tuple(im.shape))
            flat.append(im.reshape(-1))
        return cls(torch.cat(flat).contiguous(), shapes)

    def __len__(self) -> int:
        return len(self.shapes)

    def __getitem__(self, i: int) -> Tensor:
        h, w = self.shapes[i]
        o = self.offsets[i]
        return self.data[o:o + h * w].view(h, w)

    def images(self) -> list[Tensor]:
        return [self[i] for i in range(len(self))]

    @property
    def device(self):
        return self.data.device

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def numel(self) -> int:
        return sum(h * w for h, w in self.shapes)

    @property
    def plan(self) -> Tensor:
        """Device descriptor table (built on first use, shared with derived batches)."""
        if self._plan is None:
            if not self.data.is_cuda:
                raise ValueError("ragged operators need a CUDA RaggedBatch")
            lib = _lib.load()
            n = len(self.shapes)
            nbytes = lib.tm_ragged_plan_size(n)
            plan = torch.empty(int(nbytes), dtype=torch.uint8, device=self.data.device)
            with torch.cuda.device(self.data.device):
                _lib.check(lib.tm_ragged_plan(n, _lib.i64_array([h for h, _ in self.shapes]),
                                              _lib.i64_array([w for _, w in self.shapes]),
                                              _lib.i64_array(self.offsets), _lib.ptr(plan), nbytes,
                                              _lib.stream_of(self.data.device)), "tm_ragged_plan")
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
    struct, fp = _resolve_element(2, size, footprint, structure)
    o = _normalize_origin(origin, 2)
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
    """Per-image grey erosion of a float32 RaggedBatch, one launch for all images."""
    return _grey("tm_ragged_grey_erosion", batch, size, footprint, structure, mode, cval, origin, output)


def grey_dilation(batch: RaggedBatch, size=None, footprint=None, structure=None, mode="reflect", cval=0.0,
                  origin=0, output: RaggedBatch | None = None) -> RaggedBatch:
    """Per-image grey dilation of a float32 RaggedBatch, one launch for all images."""
    return _grey("tm_ragged_grey_dilation", batch, size, footprint, structure, mode, cval, origin, output)


def grey_opening(batch, size=None, footprint=None, structure=None, mode="reflect", cval=0.0, origin=0):
    tmp = grey_erosion(batch, size, footprint, structure, mode, cval, origin)
    return grey_dilation(tmp, size, footprint, structure, mode, cval, origin)


def grey_closing(batch, size=None, footprint=None, structure=None, mode="reflect", cval=0.0, origin=0):
    tmp = grey_dilation(batch, size, footprint, structure, mode, cval, origin)
    return grey_erosion(tmp, size, footprint, structure, mode, cval, origin)


def _binary(name, batch, structure, border_value, origin, output):
    _check_batch(batch, torch.bool, name)
    if structure is None:
        structure = generate_binary_structure(2, 1)
    if structure.ndim != 2:
        raise ValueError(f"structure dimension is not 2, got {structure.ndim}")
    st = (structure != 0).detach().to(device="cpu", dtype=torch.bool).contiguous()
    o = _normalize_origin(origin, 2)
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
    """Per-image binary erosion (one iteration, no mask) of a bool RaggedBatch."""
    return _binary("tm_ragged_binary_erosion", batch, structure, border_value, origin, output)


def binary_dilation(batch: RaggedBatch, structure=None, border_value=False, origin=0,
                    output: RaggedBatch | None = None) -> RaggedBatch:
    """Per-image binary dilation (one iteration, no mask) of a bool RaggedBatch."""
    return _binary("tm_ragged_binary_dilation", batch, structure, border_value, origin, output)


def binary_opening(batch, structure=None, border_value=False, origin=0):
    return binary_dilation(binary_erosion(batch, structure, border_value, origin), structure, border_value,
                           origin)


def binary_closing(batch, structure=None, border_value=False, origin=0):
    return binary_erosion(binary_dilation(batch, structure, border_value, origin), structure, border_value,
                          origin)


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
