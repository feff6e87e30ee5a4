"""CPU oracle for the torchmorph hot path -- TEST INFRASTRUCTURE ONLY.

numpy front end over ``tm_oracle.c`` (a plain-C restatement of the
reference algorithms, each function citing the reference file it follows).
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package: it is the checker, never the thing that is
measured or shipped.  The product package ``torchmorph_gb300`` does not import
it and has no CPU fallback.

The C file is built with ``gcc`` into ``oracle/build/`` by :func:`build`.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "build")
_LIB_PATH = os.path.join(_BUILD, "libtmoracle.so")
_lib = None

I64P = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    """Compile ``tm_oracle.c`` with gcc (OpenMP) into ``oracle/build``."""
    src = os.path.join(_HERE, "tm_oracle.c")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(_HERE, "tm_oracle.h"))
    ):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run(
        ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=gnu11", src, "-o", tmp, "-lm"],
        check=True,
    )
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(_LIB_PATH)
        c_i64, c_int, c_void = ctypes.c_int64, ctypes.c_int, ctypes.c_void_p
        lib.tmo_grey.argtypes = [c_int, c_void, c_void, c_i64, c_int, I64P, c_void, c_void, I64P,
                                 I64P, c_int, ctypes.c_float, c_int]
        lib.tmo_binary.argtypes = [c_int, c_void, c_void, c_i64, c_int, I64P, c_void, I64P, I64P,
                                   c_int, c_int]
        lib.tmo_edt.argtypes = [c_void, c_i64, c_int, I64P, c_void, c_void, c_void, c_void, c_int]
        lib.tmo_cdt.argtypes = [c_void, c_i64, c_int, I64P, c_int, c_void, c_void, c_int]
        lib.tmo_bfdt.argtypes = [c_void, c_i64, c_int, I64P, c_int, c_void, c_int, c_void, c_void,
                                 c_int]
        lib.tmo_sinkhorn.argtypes = [c_void, c_void, c_void, c_i64, c_i64, c_i64, ctypes.c_double,
                                     c_i64, ctypes.c_double, c_int, c_void, c_void, c_int]
        lib.tmo_sinkhorn.restype = c_i64
        lib.tmo_sinkhorn_cost.argtypes = [c_void, c_void, c_void, c_i64, c_i64, c_i64,
                                          ctypes.c_double, c_void, c_void, c_void, c_int]
        _lib = lib
    return _lib


def _i64(values):
    arr = (ctypes.c_int64 * max(1, len(values)))(*[int(v) for v in values])
    return arr


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _split(x):
    """(B, C, *S) -> batch, spatial shape."""
    x = np.asarray(x)
    return int(np.prod(x.shape[:2])), tuple(int(s) for s in x.shape[2:])


MODES = {"constant": 0, "reflect": 1, "nearest": 2, "mirror": 3, "wrap": 4}


def grey(x, structure, footprint=None, origin=None, mode="reflect", cval=0.0, dilation=False,
         nthreads=0):
    """Grey erosion/dilation of a (B, C, *S) float32 array (reference grey_kernel.cu)."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    batch, shape = _split(x)
    st = np.ascontiguousarray(structure, dtype=np.float32)
    fp = None if footprint is None else np.ascontiguousarray(footprint, dtype=np.uint8)
    origin = [0] * len(shape) if origin is None else list(origin)
    out = np.empty_like(x)
    rc = _load().tmo_grey(int(dilation), _ptr(x), _ptr(out), batch, len(shape), _i64(shape),
                          _ptr(st), _ptr(fp), _i64(st.shape), _i64(origin),
                          MODES[mode] if isinstance(mode, str) else int(mode), float(cval),
                          nthreads)
    if rc != 0:
        raise ValueError(f"tmo_grey failed ({rc})")
    return out


def binary(x, structure, origin=None, border_value=False, dilation=False, nthreads=0):
    """Binary erosion/dilation of a (B, C, *S) array (reference binary_kernel.cu)."""
    x = np.ascontiguousarray(np.asarray(x) != 0, dtype=np.uint8)
    batch, shape = _split(x)
    st = np.ascontiguousarray(np.asarray(structure) != 0, dtype=np.uint8)
    origin = [0] * len(shape) if origin is None else list(origin)
    out = np.empty_like(x)
    rc = _load().tmo_binary(int(dilation), _ptr(x), _ptr(out), batch, len(shape), _i64(shape),
                            _ptr(st), _i64(st.shape), _i64(origin), int(bool(border_value)),
                            nthreads)
    if rc != 0:
        raise ValueError(f"tmo_binary failed ({rc})")
    return out.astype(bool)


def edt(x, sampling=None, nthreads=0):
    """Exact EDT of (B, C, *S): returns (sqdist int64 | None, dist float64, indices int32)."""
    fg = np.ascontiguousarray(np.asarray(x) != 0, dtype=np.uint8)
    batch, shape = _split(fg)
    nd = len(shape)
    samp = None if sampling is None else np.ascontiguousarray(sampling, dtype=np.float64)
    sq = None if samp is not None else np.empty(fg.shape, np.int64)
    dist = np.empty(fg.shape, np.float64)
    ind = np.empty((nd,) + fg.shape, np.int32)
    rc = _load().tmo_edt(_ptr(fg), batch, nd, _i64(shape), _ptr(samp), _ptr(sq), _ptr(dist),
                         _ptr(ind), nthreads)
    if rc != 0:
        raise ValueError(f"tmo_edt failed ({rc})")
    return sq, dist, ind


CDT_METRICS = {"chessboard": 0, "taxicab": 1, "chamfer345": 2}


def cdt(x, metric="chessboard", nthreads=0):
    """Raster two-pass chamfer DT of (B, C, *S): returns (int32 cost, int32 indices)."""
    fg = np.ascontiguousarray(np.asarray(x) != 0, dtype=np.uint8)
    batch, shape = _split(fg)
    nd = len(shape)
    dist = np.empty(fg.shape, np.int32)
    ind = np.empty((nd,) + fg.shape, np.int32)
    rc = _load().tmo_cdt(_ptr(fg), batch, nd, _i64(shape), CDT_METRICS[metric], _ptr(dist),
                         _ptr(ind), nthreads)
    if rc != 0:
        raise ValueError(f"tmo_cdt failed ({rc})")
    return dist, ind


BF_METRICS = {"euclidean": 0, "taxicab": 1, "chessboard": 2}


def bfdt(x, metric="euclidean", sampling=None, return_indices=True, nthreads=0):
    """Brute-force DT of (B, C, *S): returns (float64 dist, int32 indices)."""
    fg = np.ascontiguousarray(np.asarray(x) != 0, dtype=np.uint8)
    batch, shape = _split(fg)
    nd = len(shape)
    samp = None if sampling is None else np.ascontiguousarray(sampling, dtype=np.float64)
    dist = np.empty(fg.shape, np.float64)
    ind = np.zeros((nd,) + fg.shape, np.int32)
    rc = _load().tmo_bfdt(_ptr(fg), batch, nd, _i64(shape), BF_METRICS[metric], _ptr(samp),
                          int(bool(return_indices)), _ptr(dist), _ptr(ind), nthreads)
    if rc != 0:
        raise ValueError(f"tmo_bfdt failed ({rc})")
    return dist, ind


def sinkhorn(a, b, cost, eps, max_iter, threshold=0.0, log_space=True, nthreads=0):
    """float64 Sinkhorn (reference optimal_transport.py:71-125).

    a (n, d1), b (n, d2), cost (d1, d2).  Returns (log_u, log_v, iterations run).
    """
    a = np.ascontiguousarray(a, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    c = np.ascontiguousarray(cost, np.float64)
    n, d1 = a.shape
    d2 = b.shape[1]
    lu = np.empty((n, d1))
    lv = np.empty((n, d2))
    its = _load().tmo_sinkhorn(_ptr(a), _ptr(b), _ptr(c), n, d1, d2, float(eps), int(max_iter),
                               float(threshold), int(bool(log_space)), _ptr(lu), _ptr(lv),
                               nthreads)
    return lu, lv, int(its)


def sinkhorn_cost(cost, log_u, log_v, eps, nthreads=0):
    """<P, C> and the row/column marginals of P = exp(log_u - C/eps + log_v)."""
    c = np.ascontiguousarray(cost, np.float64)
    lu = np.ascontiguousarray(log_u, np.float64)
    lv = np.ascontiguousarray(log_v, np.float64)
    n, d1 = lu.shape
    d2 = lv.shape[1]
    dist = np.empty(n)
    rm = np.empty((n, d1))
    cm = np.empty((n, d2))
    _load().tmo_sinkhorn_cost(_ptr(c), _ptr(lu), _ptr(lv), n, d1, d2, float(eps), _ptr(dist),
                              _ptr(rm), _ptr(cm), nthreads)
    return dist, rm, cm


# ------------------------------------------------ grey morphology gradient
# numpy restatement (small cases): the forward with the first extremum tap
# recorded, and the gradient routed to that tap's input voxel.  Taps follow
# torchmorph/csrc/grey_kernel.cu:271-291 (erosion reads x + delta, dilation
# x - delta, delta = k - (size // 2 + origin)); borders follow map_coord
# (grey_kernel.cu:63-97).  There is no gradient in the reference; the tie
# rule (first tap in footprint raster order) is the one the GB300 backward
# documents.

_MODES = {"constant": 0, "reflect": 1, "nearest": 2, "mirror": 3, "wrap": 4}


def map_coords(c, n, mode):
    """Border mapping of integer coordinates; -1 where the constant is used."""
    c = np.asarray(c, dtype=np.int64)
    if mode == "constant":
        return np.where((c >= 0) & (c < n), c, -1)
    if mode == "nearest":
        return np.clip(c, 0, n - 1)
    if mode == "reflect":
        r = np.mod(c, 2 * n)
        return np.where(r >= n, 2 * n - 1 - r, r)
    if mode == "mirror":
        if n == 1:
            return np.zeros_like(c)
        p = 2 * (n - 1)
        r = np.mod(c, p)
        return np.where(r >= n, p - r, r)
    if mode == "wrap":
        return np.mod(c, n)
    raise ValueError(mode)


def _grey_taps(structure, footprint, origin, dilation):
    s = np.asarray(structure)
    fp = np.ones(s.shape, bool) if footprint is None else np.asarray(footprint, bool)
    origin = [0] * s.ndim if origin is None else list(origin)
    taps = []
    for k in np.ndindex(*s.shape):
        if not fp[k]:
            continue
        delta = [k[d] - (s.shape[d] // 2 + origin[d]) for d in range(s.ndim)]
        taps.append(([-v for v in delta] if dilation else delta, s[k]))
    return taps


def grey_arg(x, structure, footprint=None, origin=None, mode="reflect", cval=0.0, dilation=False):
    """(out, arg) of grey erosion/dilation of a (B, C, *S) array in x's float dtype:
    arg = index of the first active tap (raster order) attaining the extremum, 255 if none."""
    x = np.asarray(x)
    dt = x.dtype
    shape = x.shape[2:]
    grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    best = np.full(x.shape, -np.inf if dilation else np.inf, dt)
    arg = np.full(x.shape, 255, np.uint8)
    for t, (off, val) in enumerate(_grey_taps(structure, footprint, origin, dilation)):
        idx = [map_coords(g + o, n, mode) for g, o, n in zip(grids, off, shape)]
        valid = np.logical_and.reduce([i >= 0 for i in idx])
        safe = tuple(np.where(valid, i, 0) for i in idx)
        v = np.where(valid, x[(slice(None), slice(None)) + safe], dt.type(cval)).astype(dt)
        v = (v + dt.type(val)) if dilation else (v - dt.type(val))
        better = (v > best) if dilation else (v < best)
        best = np.where(better, v, best)
        arg = np.where(better, np.uint8(t), arg)
    return best, arg


def grey_backward(grad_out, arg, structure_shape, footprint=None, origin=None, mode="reflect",
                  dilation=False):
    """float64 input gradient: each output's gradient added to the voxel its recorded tap read."""
    g = np.asarray(grad_out, np.float64)
    shape = g.shape[2:]
    gin = np.zeros_like(g)
    grids = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    taps = _grey_taps(np.zeros(structure_shape), footprint, origin, dilation)
    b_idx, c_idx = np.meshgrid(np.arange(g.shape[0]), np.arange(g.shape[1]), indexing="ij")
    for t, (off, _) in enumerate(taps):
        idx = [map_coords(gr + o, n, mode) for gr, o, n in zip(grids, off, shape)]
        valid = np.logical_and.reduce([i >= 0 for i in idx])
        sel = (arg == t) & valid[None, None]
        bb, cc, *pos = np.nonzero(sel)
        tgt = tuple(idx[d][tuple(pos)] for d in range(len(shape)))
        np.add.at(gin, (bb, cc) + tgt, g[sel])
    return gin


# ------------------------------------------------- point-cloud Sinkhorn
def _lse(z, axis):
    m = np.max(z, axis=axis, keepdims=True)
    m = np.where(np.isfinite(m), m, 0.0)
    return np.squeeze(m, axis) + np.log(np.sum(np.exp(z - m), axis=axis))


def pointcloud_sinkhorn(x, y, eps, max_iter, threshold=0.0, check_every=10, log_a=None, log_b=None):
    """float64 log-domain Sinkhorn between two point clouds (squared-Euclidean cost):
    the reference's _log_iterations (optimal_transport.py:96-125) in dual-potential form,
    f = eps (log_u - log a), g = eps (log_v - log b), started from the reference's
    log_u = log_v = 0.  Stops after the first multiple of `check_every` iterations whose
    g-update moved the column marginals of (f, g_old) by an L1 of <= threshold.
    Returns (f, g, iterations, regularised cost <f, a> + <g, b>)."""
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    n, m = len(x), len(y)
    la = np.full(n, -np.log(n)) if log_a is None else np.asarray(log_a, np.float64)
    lb = np.full(m, -np.log(m)) if log_b is None else np.asarray(log_b, np.float64)
    C = ((x[:, None] - y[None]) ** 2).sum(-1)
    f = -eps * la
    g = -eps * lb
    it = 0
    while it < max_iter:
        f = -eps * _lse((g[None] - C) / eps + lb[None], 1)
        g_new = -eps * _lse((f[:, None] - C) / eps + la[:, None], 0)
        it += 1
        check = it % check_every == 0 or it == max_iter
        err = np.sum(np.exp(lb) * np.abs(np.expm1((g - g_new) / eps))) if check else None
        g = g_new
        if check and threshold > 0 and err <= threshold:
            break
    cost = np.sum(np.exp(la) * f) + np.sum(np.exp(lb) * g)
    return f, g, it, cost
