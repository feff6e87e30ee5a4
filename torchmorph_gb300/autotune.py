"""Autotuner: per (operator, work class, device) implementation variants.

libtmcore keeps, for four operators, a table of implementation variants
indexed by a work class (``tm_tune_*`` in include/torchmorph_gb300.h):

* ``grey_flat2d``   flat 1-D / 2-D grey and binary boxes: TMA-staged
  persistent tiles at full occupancy, plain loads one CTA per tile, or TMA
  tiles with at most 1 / 2 CTAs per SM (class: log2 of the voxel count);
* ``sinkhorn_f32``  FP32 Sinkhorn: 16 or 64 histogram pairs per tile, one or
  two CTAs per SM (class from the pair count and the point count);
* ``edt_3d``        3-D exact EDT: bitmap shell search first, or the separable
  passes alone (class: log2 of the voxel count);
* ``cdt_3d``        3-D chamfer distances: bitmap shell search first (persistent
  warps on a unit queue, or one CTA per 32-row block), or the raster passes alone.

Every variant of an operator computes bit-identical results, so tuning
changes speed only.  :func:`tune` times every variant of one call with CUDA
events, checks that all of them return the same bits as the built-in choice,
keeps the fastest for the call's work class and records it in a JSON cache
keyed by device name (``$TORCHMORPH_GB300_TUNING`` or
``~/.cache/torchmorph_gb300/tuning.json``).  :func:`apply_cache` installs
the cached choices for a device; the package calls it when the library is
first loaded.  The reference has no tuner: its block sizes are compile-time
constants (torchmorph/csrc/ot_kernel.cu:9, torchmorph/csrc/edt_kernel.cu:20).
"""

from __future__ import annotations

import json
import os
import tempfile
from typing import Callable, Dict, Optional, Sequence

import torch

from . import _lib

OPS = {"grey_flat2d": 0, "sinkhorn_f32": 1, "edt_3d": 2, "cdt_3d": 3}
CACHE_VERSION = 1


def cache_path() -> str:
    path = os.environ.get("TORCHMORPH_GB300_TUNING")
    if path:
        return path
    return os.path.join(os.path.expanduser("~"), ".cache", "torchmorph_gb300", "tuning.json")


def load_cache(path: Optional[str] = None) -> Dict:
    """The cache as {"version": 1, "devices": {name: {op: {class: variant}}}}; empty if absent
    or unreadable."""
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
    except (OSError, ValueError):
        return {"version": CACHE_VERSION, "devices": {}}
    if not isinstance(data, dict) or data.get("version") != CACHE_VERSION or not isinstance(
            data.get("devices"), dict):
        return {"version": CACHE_VERSION, "devices": {}}
    return data


def save_cache(data: Dict, path: Optional[str] = None) -> str:
    """Write the cache atomically (temporary file + rename)."""
    path = path or cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    fd, tmp = tempfile.mkstemp(dir=os.path.dirname(os.path.abspath(path)), suffix=".tmp")
    with os.fdopen(fd, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return path


def set_variant(op: str, cls: int, variant: int) -> None:
    lib = _lib.load()
    _lib.check(lib.tm_tune_set(OPS[op], int(cls), int(variant)), "tm_tune_set")


def get_variant(op: str, cls: int) -> int:
    return int(_lib.load().tm_tune_get(OPS[op], int(cls)))


def variants(op: str) -> int:
    return int(_lib.load().tm_tune_variants(OPS[op]))


def work_class(op: str, a: int, b: int = 0) -> int:
    return int(_lib.load().tm_tune_class(OPS[op], int(a), int(b)))


def apply_cache(device_name: Optional[str] = None, path: Optional[str] = None) -> int:
    """Install the cached variants of `device_name` (default: the current CUDA device);
    returns how many entries were applied.  Entries with unknown operators or
    out-of-range values are skipped."""
    if device_name is None:
        if not torch.cuda.is_available():
            return 0
        device_name = torch.cuda.get_device_name(torch.cuda.current_device())
    entries = load_cache(path)["devices"].get(device_name, {})
    applied = 0
    for op, table in entries.items():
        if op not in OPS or not isinstance(table, dict):
            continue
        for cls, variant in table.items():
            try:
                cls_i, var_i = int(cls), int(variant)
            except (TypeError, ValueError):
                continue
            if 0 <= cls_i < 64 and 0 <= var_i < variants(op):
                set_variant(op, cls_i, var_i)
                applied += 1
    return applied


def _snapshot(out) -> Sequence[torch.Tensor]:
    if isinstance(out, torch.Tensor):
        return [out.detach().clone()]
    return [t.detach().clone() for t in out if isinstance(t, torch.Tensor)]


def tune(op: str, call: Callable[[], object], a: int, b: int = 0, *, warmup: int = 2, reps: int = 5,
         persist: bool = True, path: Optional[str] = None) -> Dict:
    """Time every variant of `op` on `call()` (a call of the public operator whose work
    class is given by `a`, `b` as for :func:`work_class`), check that each returns the
    same bits as the built-in choice, keep the fastest for the class and, with
    `persist`, record it in the cache.  Returns {"class", "times_ms" (per variant),
    "builtin_ms", "best"}."""
    if op not in OPS:
        raise ValueError(f"unknown operator {op!r}; one of {sorted(OPS)}")
    cls = work_class(op, a, b)
    previous = get_variant(op, cls)
    stream = torch.cuda.current_stream()

    def timed() -> float:
        for _ in range(warmup):
            call()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        start.record(stream)
        for _ in range(reps):
            call()
        end.record(stream)
        torch.cuda.synchronize()
        return start.elapsed_time(end) / reps

    try:
        set_variant(op, cls, -1)
        reference = _snapshot(call())
        builtin_ms = timed()
        times = []
        for v in range(variants(op)):
            set_variant(op, cls, v)
            got = _snapshot(call())
            if len(got) != len(reference) or not all(torch.equal(x, y) for x, y in zip(got, reference)):
                raise RuntimeError(f"{op} variant {v} differs from the built-in choice")
            times.append(timed())
    except Exception:
        set_variant(op, cls, previous)
        raise
    best = min(range(len(times)), key=times.__getitem__)
    set_variant(op, cls, best)
    if persist:
        data = load_cache(path)
        name = torch.cuda.get_device_name(torch.cuda.current_device())
        data["devices"].setdefault(name, {}).setdefault(op, {})[str(cls)] = best
        save_cache(data, path)
    return {"class": cls, "times_ms": times, "builtin_ms": builtin_ms, "best": best}


# ---------------------------------------------------------------- helpers
def tune_grey_dilation(x: torch.Tensor, size=3, **kw) -> Dict:
    """Tune the flat-box path on a grey_dilation call of `x` (B, C, H, W)."""
    from . import grey_dilation

    return tune("grey_flat2d", lambda: grey_dilation(x, size=size), x.numel(), **kw)


def tune_edt(x: torch.Tensor, return_indices: bool = True, **kw) -> Dict:
    """Tune the 3-D EDT on a call of `x` (B, C, D, H, W)."""
    from . import euclidean_distance_transform

    return tune("edt_3d", lambda: euclidean_distance_transform(x, return_indices=return_indices),
                x.numel(), **kw)


def tune_cdt(x: torch.Tensor, metric: str = "chessboard", **kw) -> Dict:
    """Tune the 3-D chamfer distances (no indices) on a call of `x`."""
    from . import chamfer_distance_transform

    return tune("cdt_3d", lambda: chamfer_distance_transform(x, metric=metric), x.numel(), **kw)


def tune_sinkhorn(a: torch.Tensor, b: torch.Tensor, cost: torch.Tensor, epsilon: float, max_iter: int = 20,
                  log_space: bool = False, **kw) -> Dict:
    """Tune the FP32 Sinkhorn solver on `max_iter` iterations of (a, b, cost)."""
    from . import _C

    def call():
        return _C.sinkhorn_f32_solve(a, b, cost, epsilon, max_iter, 0.0, log_space)[:2]

    return tune("sinkhorn_f32", call, a.shape[0], a.shape[1], **kw)
