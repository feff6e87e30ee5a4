"""Drop-in for the reference's pybind11 module ``torchmorph._C``.

Same nine function names, argument meaning, return values and error type
(``RuntimeError``) as torchmorph/csrc/torchmorph.cpp:79-155, implemented as
thin adapters that turn tensors into pointers/sizes and call the C ABI of
libtmcore.so on the input device's current stream.  Outputs are allocated
through PyTorch's caching allocator, as in the reference.
"""

from __future__ import annotations

import ctypes

import torch

from . import _lib

_TORCH_TO_TM = {torch.float32: _lib.TM_F32, torch.bool: _lib.TM_U8, torch.uint8: _lib.TM_U8}


def _require(cond: bool, msg: str) -> None:
    if not cond:
        raise RuntimeError(msg)


def _batch_shape(t: torch.Tensor):
    _require(t.dim() >= 3, "input must be (B, C, spatial...) with at least 3 dimensions")
    return t.shape[0] * t.shape[1], list(t.shape[2:])


def _host_f32(t: torch.Tensor):
    return ctypes.cast(t.data_ptr(), _lib.F32P)


def _host_u8(t: torch.Tensor):
    return ctypes.cast(t.data_ptr(), _lib.U8P)


def _workspace(nbytes: int, device) -> torch.Tensor | None:
    if nbytes == 0:
        return None
    return torch.empty(int(nbytes), dtype=torch.uint8, device=device)


# ------------------------------------------------------------------- grey
def _grey(fn_name, input, structure, footprint, origin, mode, cval):
    _require(input.is_cuda, "input must be a CUDA tensor")
    _require(not structure.is_cuda, "structure must be a CPU tensor")
    _require(not footprint.is_cuda, "footprint must be a CPU tensor")
    _require(input.is_contiguous(), "input must be contiguous")
    _require(structure.is_contiguous(), "structure must be contiguous")
    _require(footprint.is_contiguous(), "footprint must be contiguous")
    _require(input.dtype == torch.float32, "input must be float32")
    _require(structure.dtype == torch.float32, "structure must be float32")
    _require(footprint.dtype == torch.bool, "footprint must be bool")
    nd = structure.dim()
    _require(0 < nd <= 8, f"structure dimension must be in 1-8, got {nd}")
    _require(len(origin) == nd, "origin length must match structure dimensions")
    _require(input.dim() == nd + 2, "input spatial dimensions must match structure dimensions")
    use_fp = footprint.numel() != 0
    if use_fp:
        _require(tuple(footprint.shape) == tuple(structure.shape),
                 "footprint shape must match structure shape")
    batch, shape = _batch_shape(input)
    out = torch.empty_like(input)
    lib = _lib.load()
    with torch.cuda.device(input.device):
        st = getattr(lib, fn_name)(
            _lib.ptr(input), _lib.ptr(out), batch, nd, _lib.i64_array(shape), _host_f32(structure),
            _host_u8(footprint) if use_fp else None, _lib.i64_array(structure.shape),
            _lib.i64_array(origin), int(mode), float(cval), _lib.stream_of(input.device))
    _lib.check(st, fn_name)
    return out


def grey_erosion_cuda(input, structure, footprint, origin, mode, cval):
    """N-dimensional fused grey erosion (reference grey_kernel.cu:332-343)."""
    return _grey("tm_grey_erosion", input, structure, footprint, origin, mode, cval)


def grey_dilation_cuda(input, structure, footprint, origin, mode, cval):
    """N-dimensional fused grey dilation (reference grey_kernel.cu:345-356)."""
    return _grey("tm_grey_dilation", input, structure, footprint, origin, mode, cval)


_TM_ERR_UNSUPPORTED = 2


_COMPOSITES = {"gradient": "tm_grey_gradient", "laplace": "tm_grey_laplace", "opening": "tm_grey_opening",
               "closing": "tm_grey_closing", "white_tophat": "tm_white_tophat",
               "black_tophat": "tm_black_tophat"}


def grey_composite(kind, input, structure, footprint, origin, mode, cval):
    """One-pass composite of a batch (tm_grey_gradient, tm_grey_laplace: 2-D items;
    tm_grey_opening / closing, tm_white_tophat / black_tophat: 1-D or 2-D items with flat
    boxes up to 33 per axis); None when the element is outside the one-pass kernel's
    limits, so that the caller composes the operators instead."""
    _require(input.is_cuda and input.is_contiguous() and input.dtype == torch.float32,
             "input must be a contiguous float32 CUDA tensor")
    nd = structure.dim()
    _require(len(origin) == nd and input.dim() == nd + 2, "structure/origin/input dimensions disagree")
    name = _COMPOSITES[kind]
    if nd != 2 and not (nd == 1 and kind not in ("gradient", "laplace")):
        return None
    use_fp = footprint.numel() != 0
    batch, shape = _batch_shape(input)
    out = torch.empty_like(input)
    lib = _lib.load()
    with torch.cuda.device(input.device):
        st = getattr(lib, name)(
            _lib.ptr(input), _lib.ptr(out), batch, nd, _lib.i64_array(shape), _host_f32(structure),
            _host_u8(footprint) if use_fp else None, _lib.i64_array(structure.shape),
            _lib.i64_array(origin), int(mode), float(cval), _lib.stream_of(input.device))
    if st == _TM_ERR_UNSUPPORTED:
        return None
    _lib.check(st, name)
    return out


def _grey_arg(fn_name, input, structure, footprint, origin, mode, cval):
    """(output, argument) of the forward with the first extremum tap recorded per output."""
    _require(input.is_cuda and input.is_contiguous() and input.dtype == torch.float32,
             "input must be a contiguous float32 CUDA tensor")
    nd = structure.dim()
    _require(len(origin) == nd and input.dim() == nd + 2, "structure/origin/input dimensions disagree")
    use_fp = footprint.numel() != 0
    batch, shape = _batch_shape(input)
    out = torch.empty_like(input)
    arg = torch.empty(input.shape, dtype=torch.uint8, device=input.device)
    lib = _lib.load()
    with torch.cuda.device(input.device):
        st = getattr(lib, fn_name)(
            _lib.ptr(input), _lib.ptr(out), _lib.ptr(arg), batch, nd, _lib.i64_array(shape),
            _host_f32(structure), _host_u8(footprint) if use_fp else None,
            _lib.i64_array(structure.shape), _lib.i64_array(origin), int(mode), float(cval),
            _lib.stream_of(input.device))
    _lib.check(st, fn_name)
    return out, arg


def grey_erosion_arg(input, structure, footprint, origin, mode, cval):
    return _grey_arg("tm_grey_erosion_arg", input, structure, footprint, origin, mode, cval)


def grey_dilation_arg(input, structure, footprint, origin, mode, cval):
    return _grey_arg("tm_grey_dilation_arg", input, structure, footprint, origin, mode, cval)


def grey_morphology_backward(grad_output, arg, sshape, footprint, origin, mode, dilation):
    """grad_input of grey erosion/dilation from grad_output and the recorded argument."""
    g = grad_output.contiguous().float()
    _require(g.is_cuda and arg.is_cuda and arg.shape == g.shape, "grad_output/argument mismatch")
    nd = len(sshape)
    batch, shape = _batch_shape(g)
    gin = torch.empty_like(g)
    use_fp = footprint.numel() != 0
    name = "tm_grey_dilation_backward" if dilation else "tm_grey_erosion_backward"
    lib = _lib.load()
    with torch.cuda.device(g.device):
        st = getattr(lib, name)(
            _lib.ptr(g), _lib.ptr(arg), _lib.ptr(gin), batch, nd, _lib.i64_array(shape),
            _host_u8(footprint) if use_fp else None, _lib.i64_array(sshape), _lib.i64_array(origin),
            int(mode), _lib.stream_of(g.device))
    _lib.check(st, name)
    return gin


# ----------------------------------------------------------------- binary
def _binary(fn_name, input, structure, origin, border_value, out=None):
    _require(input.is_cuda, "input must be a CUDA tensor")
    _require(not structure.is_cuda, "structure must be a CPU tensor")
    _require(input.is_contiguous(), "input must be contiguous")
    _require(structure.is_contiguous(), "structure must be contiguous")
    _require(input.dtype == torch.bool, "input must be bool")
    _require(structure.dtype == torch.bool, "structure must be bool")
    nd = structure.dim()
    _require(0 < nd <= 8, f"structure dimension must be in 1-8, got {nd}")
    _require(len(origin) == nd, "origin length must match structure dimensions")
    _require(input.dim() == nd + 2, "input spatial dimensions must match structure dimensions")
    batch, shape = _batch_shape(input)
    if out is None:
        out = torch.empty_like(input)
    lib = _lib.load()
    with torch.cuda.device(input.device):
        st = getattr(lib, fn_name)(
            _lib.ptr(input), _lib.ptr(out), batch, nd, _lib.i64_array(shape), _host_u8(structure),
            _lib.i64_array(structure.shape), _lib.i64_array(origin), int(bool(border_value)),
            _lib.stream_of(input.device))
    _lib.check(st, fn_name)
    return out


def binary_composite(kind, input, structure, origin, border_value):
    """One-pass binary opening / closing (one iteration) of 1-D / 2-D items on bit-packed
    tiles (tm_binary_opening / tm_binary_closing); None when the structure is beyond the
    kernel's limits, so that the caller composes the operators."""
    name = {"opening": "tm_binary_opening", "closing": "tm_binary_closing"}[kind]
    if structure.dim() > 2:
        return None
    out = torch.empty_like(input)
    try:
        return _binary(name, input, structure, origin, border_value, out)
    except _lib.TorchmorphError as e:
        if e.status == _TM_ERR_UNSUPPORTED:
            return None
        raise


def binary_erosion_cuda(input, structure, origin, border_value):
    """N-dimensional fused binary erosion (reference binary_kernel.cu:252-261)."""
    return _binary("tm_binary_erosion", input, structure, origin, border_value)


def binary_dilation_cuda(input, structure, origin, border_value):
    """N-dimensional fused binary dilation (reference binary_kernel.cu:263-272)."""
    return _binary("tm_binary_dilation", input, structure, origin, border_value)


# ------------------------------------------------------ distance transforms
def _dt_input(input):
    _require(input.is_cuda, "Input must be a CUDA tensor")
    _require(input.dtype in _TORCH_TO_TM, "Input must be float32 or bool")
    input = input.contiguous()
    batch, shape = _batch_shape(input)
    return input, batch, shape


def edt(input, sampling=None, return_distances=True, return_indices=False, sqdist=False,
        distances_out=None, indices_out=None):
    """EDT through tm_edt; input float32 (nonzero = foreground) or bool.

    Returns (distances | None, indices | None, squared | None).  Preallocated
    float32/int32 outputs may be passed to skip allocation.
    """
    input, batch, shape = _dt_input(input)
    nd = len(shape)
    if sampling is not None and len(sampling) == 0:
        sampling = None
    if sampling is not None:
        _require(len(sampling) == nd, "sampling length must match spatial dimensions")
    dev = input.device
    dist = None
    if return_distances:
        dist = distances_out if distances_out is not None else torch.empty(
            input.shape, dtype=torch.float32, device=dev)
    ind = None
    if return_indices:
        ind = indices_out if indices_out is not None else torch.empty(
            (nd, *input.shape), dtype=torch.int32, device=dev)
    sq = torch.empty(input.shape, dtype=torch.int32, device=dev) if sqdist else None
    lib = _lib.load()
    with torch.cuda.device(dev):
        shp = _lib.i64_array(shape)
        samp = None if sampling is None else _lib.f32_array(sampling)
        ws = _workspace(lib.tm_edt_workspace_size(batch, nd, shp, samp), dev)
        st = lib.tm_edt(_lib.ptr(input), _TORCH_TO_TM[input.dtype], batch, nd, shp, samp, _lib.ptr(dist),
                        _lib.ptr(ind), _lib.ptr(sq), _lib.ptr(ws),
                        0 if ws is None else ws.numel(), _lib.stream_of(dev))
    _lib.check(st, "tm_edt")
    return dist, ind, sq


def edt_cuda(input, sampling, return_distances=True, return_indices=False):
    """Exact EDT (reference edt_kernel.cu:904-958); returns (distances, indices | None)."""
    dist, ind, _ = edt(input, sampling, True, return_indices)
    return dist, ind


_CDT_METRICS = {"chessboard": 0, "taxicab": 1, "chamfer345": 2}


def cdt(input, metric="chessboard", return_distances=True, return_indices=False,
        distances_out=None, indices_out=None):
    input, batch, shape = _dt_input(input)
    _require(metric in _CDT_METRICS, "metric must be 'chessboard' or 'taxicab'")
    _require(return_distances or return_indices,
             "At least one of return_distances or return_indices must be True")
    nd = len(shape)
    dev = input.device
    dist = None
    if return_distances:
        dist = distances_out if distances_out is not None else torch.empty(
            input.shape, dtype=torch.float32, device=dev)
    ind = None
    if return_indices:
        ind = indices_out if indices_out is not None else torch.empty(
            (nd, *input.shape), dtype=torch.int32, device=dev)
    lib = _lib.load()
    with torch.cuda.device(dev):
        shp = _lib.i64_array(shape)
        ws = _workspace(lib.tm_cdt_workspace_size(batch, nd, shp), dev)
        st = lib.tm_cdt(_lib.ptr(input), _TORCH_TO_TM[input.dtype], batch, nd, shp,
                        _CDT_METRICS[metric], _lib.ptr(dist), _lib.ptr(ind), _lib.ptr(ws),
                        0 if ws is None else ws.numel(), _lib.stream_of(dev))
    _lib.check(st, "tm_cdt")
    return dist, ind


def cdt_cuda(input, metric="chessboard", return_distances=True, return_indices=False):
    """Chamfer DT (reference cdt_kernel.cu:269-463); returns (distances | None, indices | None)."""
    return cdt(input, metric, return_distances, return_indices)


_BF_METRICS = {"euclidean": 0, "taxicab": 1, "chessboard": 2}


def bfdt(input, metric="euclidean", sampling=None, return_distances=True, return_indices=False,
         distances_out=None, indices_out=None):
    input, batch, shape = _dt_input(input)
    _require(metric in _BF_METRICS,
             "Unsupported metric type. Use 'euclidean', 'taxicab', or 'chessboard'.")
    nd = len(shape)
    if sampling is not None and len(sampling) == 0:
        sampling = None
    if sampling is not None:
        _require(len(sampling) == nd, "sampling length must match spatial dimensions")
    dev = input.device
    dist = None
    if return_distances:
        dist = distances_out if distances_out is not None else torch.empty(
            input.shape, dtype=torch.float32, device=dev)
    ind = None
    if return_indices:
        ind = indices_out if indices_out is not None else torch.empty(
            (nd, *input.shape), dtype=torch.int32, device=dev)
    lib = _lib.load()
    with torch.cuda.device(dev):
        shp = _lib.i64_array(shape)
        ws = _workspace(lib.tm_bfdt_workspace_size(batch, nd, shp), dev)
        st = lib.tm_bfdt(_lib.ptr(input), _TORCH_TO_TM[input.dtype], batch, nd, shp,
                         _BF_METRICS[metric], None if sampling is None else _lib.f32_array(sampling),
                         _lib.ptr(dist), _lib.ptr(ind), _lib.ptr(ws),
                         0 if ws is None else ws.numel(), _lib.stream_of(dev))
    _lib.check(st, "tm_bfdt")
    return dist, ind


def bfdt_cuda(input, metric="euclidean", sampling=(), return_distances=True, return_indices=False):
    """Brute-force DT (reference bfdt_kernel.cu:154-297); returns (distances, indices | None)."""
    dist, ind = bfdt(input, metric, list(sampling), True, return_indices)
    return dist, ind


# --------------------------------------------------------------- sinkhorn
def _ot_check(t, numel, name):
    _require(t.is_cuda, f"{name} must be a CUDA tensor")
    _require(t.dtype == torch.float32, f"{name} must be float32")
    _require(t.is_contiguous(), f"{name} must be contiguous")
    _require(t.numel() == numel, f"{name} must have {numel} elements, got {t.numel()}")


def _ot_shapes(u, mat):
    _require(mat.dim() == 2 and mat.shape[0] == mat.shape[1], "cost/kernel matrix must be square")
    _require(u.dim() == 2 and u.shape[1] == mat.shape[0],
             "scaling vectors must be (n, d) with d matching the matrix")
    return u.shape[0], u.shape[1]


def _iter_workspace(device):
    return _workspace(_lib.load().tm_sinkhorn_iter_workspace_size(), device)


def sinkhorn_fastiter(a, b, K, K_T, u, v, n_iter):
    """n_iter scaling-form iterations in place, one persistent launch
    (reference ot_kernel.cu:188-233)."""
    n, d = _ot_shapes(u, K)
    for t, name in ((a, "a"), (b, "b"), (u, "u"), (v, "v")):
        _ot_check(t, n * d, name)
    _ot_check(K, d * d, "K")
    _ot_check(K_T, d * d, "K_T")
    lib = _lib.load()
    with torch.cuda.device(u.device):
        ws = _iter_workspace(u.device)
        st = lib.tm_sinkhorn_fastiter(_lib.ptr(a), _lib.ptr(b), _lib.ptr(K), _lib.ptr(K_T),
                                      _lib.ptr(u), _lib.ptr(v), n, d, int(n_iter), _lib.ptr(ws),
                                      ws.numel(), _lib.stream_of(u.device))
    _lib.check(st, "sinkhorn_fastiter")
    return u, v


def sinkhorn_logiter(log_a, log_b, M, M_T, log_u, log_v, n_iter, epsilon):
    """n_iter log-domain iterations in place, one persistent launch
    (reference ot_kernel.cu:235-283)."""
    _require(epsilon > 0, f"epsilon must be positive, got {epsilon}")
    n, d = _ot_shapes(log_u, M)
    for t, name in ((log_a, "log_a"), (log_b, "log_b"), (log_u, "log_u"), (log_v, "log_v")):
        _ot_check(t, n * d, name)
    _ot_check(M, d * d, "M")
    _ot_check(M_T, d * d, "M_T")
    lib = _lib.load()
    with torch.cuda.device(log_u.device):
        ws = _iter_workspace(log_u.device)
        st = lib.tm_sinkhorn_logiter(_lib.ptr(log_a), _lib.ptr(log_b), _lib.ptr(M), _lib.ptr(M_T),
                                     _lib.ptr(log_u), _lib.ptr(log_v), n, d, int(n_iter),
                                     float(epsilon), _lib.ptr(ws), ws.numel(),
                                     _lib.stream_of(log_u.device))
    _lib.check(st, "sinkhorn_logiter")
    return log_u, log_v


def sinkhorn_f32_solve(a, b, cost_matrix, epsilon, max_iter, threshold=0.0, log_space=False,
                       check_every=10):
    """A whole FP32 Sinkhorn solve on the device (libtmcore tm_sinkhorn_f32_solve).

    a, b: (n, d) float32 CUDA histograms (rows summing to 1); cost_matrix (d, d), or
    None for the cost |i - j| of d points on a line, computed where it is used.
    Runs max_iter iterations in one launch, or, with threshold > 0, stops on
    the device after the first multiple of `check_every` iterations at which
    every pair's L1 row-marginal residual is <= threshold.  Returns (log_u,
    log_v, cost, row_err, iterations): fp32 (n, d) log-potentials with the
    reference's meaning, fp64 (n,) transport costs <P, C> and L1 row-marginal
    residuals of the returned potentials (no plan is materialised), and the
    iteration count as a 0-dim int32 device tensor (no host synchronisation).
    """
    _require(epsilon > 0, f"epsilon must be positive, got {epsilon}")
    _require(a.dim() == 2 and a.shape == b.shape, "a and b must be (n, d) of the same shape")
    n, d = a.shape
    for t, name in ((a, "a"), (b, "b")):
        _ot_check(t, n * d, name)
    if cost_matrix is not None:
        _ot_check(cost_matrix, d * d, "cost_matrix")
    lib = _lib.load()
    dev = a.device
    check = int(check_every) if threshold > 0 else 0
    with torch.cuda.device(dev):
        nbytes = lib.tm_sinkhorn_f32_workspace_size(n, d, int(bool(log_space)), int(max_iter), check,
                                                    int(cost_matrix is None))
        ws = _workspace(nbytes, dev)
        log_u = torch.empty((n, d), dtype=torch.float32, device=dev)
        log_v = torch.empty_like(log_u)
        cost = torch.empty(n, dtype=torch.float64, device=dev)
        row_err = torch.empty_like(cost)
        its = torch.empty((), dtype=torch.int32, device=dev)
        st = lib.tm_sinkhorn_f32_solve(_lib.ptr(a), _lib.ptr(b), _lib.ptr(cost_matrix), n, d,
                                       float(epsilon), int(bool(log_space)), int(max_iter),
                                       float(threshold), max(check, 1), _lib.ptr(log_u),
                                       _lib.ptr(log_v), _lib.ptr(cost), _lib.ptr(row_err),
                                       _lib.ptr(its), _lib.ptr(ws), nbytes, _lib.stream_of(dev))
    _lib.check(st, "sinkhorn_f32_solve")
    return log_u, log_v, cost, row_err, its


def _plan_args(log_u, log_v, cost_matrix, epsilon):
    _require(epsilon > 0, f"epsilon must be positive, got {epsilon}")
    n, d = log_u.shape
    for t, name in ((log_u, "log_u"), (log_v, "log_v")):
        _ot_check(t, n * d, name)
    if cost_matrix is not None:  # None: the line cost |i - j|
        _ot_check(cost_matrix, d * d, "cost_matrix")
    return n, d


def sinkhorn_plan(log_u, log_v, cost_matrix, epsilon):
    """(n, d, d) transport plans exp((log u - C / eps) + log v), one pass."""
    n, d = _plan_args(log_u, log_v, cost_matrix, epsilon)
    out = torch.empty((n, d, d), dtype=torch.float32, device=log_u.device)
    with torch.cuda.device(log_u.device):
        st = _lib.load().tm_sinkhorn_plan(_lib.ptr(log_u), _lib.ptr(log_v), _lib.ptr(cost_matrix), n, d,
                                          float(epsilon), _lib.ptr(out), _lib.stream_of(log_u.device))
    _lib.check(st, "sinkhorn_plan")
    return out


def sinkhorn_cost_grad(log_u, log_v, cost_matrix, epsilon, grad_distance):
    """(d, d) envelope gradient sum_b grad_distance[b] P_b, plans recomputed, never stored."""
    n, d = _plan_args(log_u, log_v, cost_matrix, epsilon)
    _ot_check(grad_distance, n, "grad_distance")
    out = torch.empty((d, d), dtype=torch.float32, device=log_u.device)
    with torch.cuda.device(log_u.device):
        st = _lib.load().tm_sinkhorn_cost_grad(_lib.ptr(log_u), _lib.ptr(log_v), _lib.ptr(cost_matrix),
                                               _lib.ptr(grad_distance), n, d, float(epsilon),
                                               _lib.ptr(out), _lib.stream_of(log_u.device))
    _lib.check(st, "sinkhorn_cost_grad")
    return out


# ----------------------------------------------- sinkhorn on tensor cores
def sinkhorn_tc_solve(a, b, cost_matrix, epsilon, max_iter, threshold=0.0, check_every=10):
    """Shared-cost batched Sinkhorn on the tensor cores (libtmcore tm_sinkhorn_tc_*).

    a, b: (n, d) float32 CUDA histograms (rows summing to 1); cost_matrix (d, d).
    Runs max_iter iterations, or stops after the first multiple of
    `check_every` iterations whose L1 row-marginal residual is <= threshold
    for every pair (threshold > 0).  Returns (log_u, log_v, cost, row_err,
    iterations): fp32 (n, d) log-potentials with the reference's meaning,
    fp64 (n,) transport costs <P, C> and L1 row-marginal residuals of the
    returned potentials, and the number of iterations run.
    """
    _require(epsilon > 0, f"epsilon must be positive, got {epsilon}")
    _require(a.dim() == 2 and a.shape == b.shape, "a and b must be (n, d) of the same shape")
    n, d = a.shape
    for t, name in ((a, "a"), (b, "b")):
        _ot_check(t, n * d, name)
    _ot_check(cost_matrix, d * d, "cost_matrix")
    lib = _lib.load()
    dev = a.device
    with torch.cuda.device(dev):
        stream = _lib.stream_of(dev)
        nbytes = lib.tm_sinkhorn_tc_workspace_size(n, d)
        ws = _workspace(nbytes, dev)
        _lib.check(lib.tm_sinkhorn_tc_init(_lib.ptr(a), _lib.ptr(b), _lib.ptr(cost_matrix), n, d,
                                           float(epsilon), _lib.ptr(ws), nbytes, stream),
                   "sinkhorn_tc_init")
        err = torch.zeros(n, dtype=torch.float64, device=dev)
        done = 0
        max_iter = int(max_iter)
        while done < max_iter:
            step = min(int(check_every), max_iter - done) if threshold > 0 else max_iter - done
            _lib.check(lib.tm_sinkhorn_tc_iterate(n, d, step, _lib.ptr(err) if threshold > 0 else None,
                                                  _lib.ptr(ws), nbytes, stream),
                       "sinkhorn_tc_iterate")
            done += step
            if threshold > 0 and err.max().item() <= threshold:
                break
        log_u = torch.empty((n, d), dtype=torch.float32, device=dev)
        log_v = torch.empty_like(log_u)
        cost = torch.empty(n, dtype=torch.float64, device=dev)
        row_err = torch.empty_like(cost)
        _lib.check(lib.tm_sinkhorn_tc_finish(n, d, _lib.ptr(log_u), _lib.ptr(log_v), _lib.ptr(cost),
                                             _lib.ptr(row_err), _lib.ptr(ws), nbytes, stream),
                   "sinkhorn_tc_finish")
    return log_u, log_v, cost, row_err, done
