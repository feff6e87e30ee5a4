"""Entropic OT between many point clouds of uneven sizes, differentiable.

:class:`PointCloudSinkhorn` solves a ragged batch of OT problems between
point clouds in R^3 with the squared-Euclidean cost, uniform (or given)
weights, all problems in ONE persistent launch (libtmcore
``tm_pointcloud_sinkhorn``): log-domain Sinkhorn iterations (the form of
the reference's ``_log_iterations``, torchmorph/optimal_transport.py:96-125,
with the cost recomputed from the points instead of a (d, d) matrix).  It
returns the regularised cost ``<f, a> + <g, b>`` per problem; its gradient
w.r.t. the points is the envelope-theorem gradient
``d/dx_i = 2 sum_j P_ij (x_i - y_j)`` computed by a hand-written kernel that
recomputes the plan entries instead of storing them.  The reference has no
ragged or point-cloud OT API.
"""

from __future__ import annotations

from typing import Sequence

import numpy as np
import torch
from torch import Tensor

from . import _lib


def pack_clouds(clouds: Sequence[Tensor]) -> tuple[Tensor, list[int]]:
    """Concatenate (k_p, 3) clouds into one (sum k_p, 3) tensor plus their sizes."""
    if len(clouds) == 0:
        raise ValueError("at least one point cloud is required")
    for c in clouds:
        if c.dim() != 2 or c.shape[1] != 3 or c.shape[0] < 1:
            raise ValueError("point clouds must be non-empty (k, 3) tensors")
    return torch.cat(list(clouds), 0), [int(c.shape[0]) for c in clouds]


def _log_weights(weights, sizes, like):
    if weights is None:  # uniform: log(1 / k) for each of a problem's k points, one copy
        k = np.asarray(sizes, dtype=np.float64)
        return torch.from_numpy(np.repeat(-np.log(k), k.astype(np.int64)).astype(np.float32)).to(like.device)
    w = weights.to(device=like.device, dtype=torch.float32).reshape(-1)
    if w.numel() != sum(sizes):
        raise ValueError("weights must have one entry per point")
    return torch.log(w).contiguous()


def _solve(x, y, la, lb, nx, ny, eps, max_iter, threshold, check_every):
    lib = _lib.load()
    P = len(nx)
    dev = x.device
    nbytes = lib.tm_pointcloud_sinkhorn_workspace_size(P, _lib.i64_array(nx), _lib.i64_array(ny), max_iter)
    ws = torch.empty(int(nbytes), dtype=torch.uint8, device=dev)
    f = torch.empty(x.shape[0], dtype=torch.float32, device=dev)
    g = torch.empty(y.shape[0], dtype=torch.float32, device=dev)
    cost = torch.empty(P, dtype=torch.float64, device=dev)
    its = torch.empty(P, dtype=torch.int32, device=dev)
    with torch.cuda.device(dev):
        _lib.check(lib.tm_pointcloud_sinkhorn(
            _lib.ptr(x), _lib.ptr(y), _lib.ptr(la), _lib.ptr(lb), P, _lib.i64_array(nx),
            _lib.i64_array(ny), float(eps), int(max_iter), float(threshold), int(check_every),
            _lib.ptr(f), _lib.ptr(g), _lib.ptr(cost), _lib.ptr(its), _lib.ptr(ws), nbytes,
            _lib.stream_of(dev)), "tm_pointcloud_sinkhorn")
    return f, g, cost, its


def _grad(x, y, la, lb, f, g, nx, ny, eps, grad_cost, need_x, need_y):
    lib = _lib.load()
    P = len(nx)
    dev = x.device
    ws = torch.empty(int(lib.tm_pointcloud_sinkhorn_grad_workspace_size(P)), dtype=torch.uint8, device=dev)
    gx = torch.empty_like(x) if need_x else None
    gy = torch.empty_like(y) if need_y else None
    scale = grad_cost.to(device=dev, dtype=torch.float32).contiguous()
    with torch.cuda.device(dev):
        _lib.check(lib.tm_pointcloud_sinkhorn_grad(
            _lib.ptr(x), _lib.ptr(y), _lib.ptr(la), _lib.ptr(lb), _lib.ptr(f), _lib.ptr(g), P,
            _lib.i64_array(nx), _lib.i64_array(ny), float(eps), _lib.ptr(scale), _lib.ptr(gx),
            _lib.ptr(gy), _lib.ptr(ws), ws.numel(), _lib.stream_of(dev)), "tm_pointcloud_sinkhorn_grad")
    return gx, gy


class _PointCloudCost(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, y, la, lb, nx, ny, eps, max_iter, threshold, check_every):
        xc, yc = x.detach().contiguous().float(), y.detach().contiguous().float()
        f, g, cost, its = _solve(xc, yc, la, lb, nx, ny, eps, max_iter, threshold, check_every)
        ctx.save_for_backward(xc, yc, la, lb, f, g)
        ctx.meta = (nx, ny, eps, x.dtype, y.dtype)
        ctx.mark_non_differentiable(f, g, its)
        return cost.to(x.dtype), f, g, its

    @staticmethod
    def backward(ctx, grad_cost, _gf, _gg, _gi):
        xc, yc, la, lb, f, g = ctx.saved_tensors
        nx, ny, eps, xdt, ydt = ctx.meta
        gx, gy = _grad(xc, yc, la, lb, f, g, nx, ny, eps, grad_cost, ctx.needs_input_grad[0],
                       ctx.needs_input_grad[1])
        return (None if gx is None else gx.to(xdt), None if gy is None else gy.to(ydt), None, None, None,
                None, None, None, None, None)


class PointCloudSinkhorn:
    """Regularised OT cost between the point-cloud pairs of a ragged batch.

    ``solver(x, y, x_sizes, y_sizes)`` with x (sum n_p, 3) and y (sum m_p, 3)
    CUDA tensors returns the (P,) regularised costs (differentiable w.r.t. x
    and y).  Each problem stops when the L1 column-marginal error of its plan
    is <= ``threshold`` (checked every ``check_every`` iterations) or after
    ``max_iter`` iterations.  ``solve`` also returns the potentials and
    iteration counts.
    """

    def __init__(self, epsilon=0.05, max_iter=1000, threshold=1e-5, check_every=10):
        if epsilon <= 0:
            raise ValueError("epsilon must be positive.")
        if max_iter <= 0:
            raise ValueError("max_iter must be positive.")
        if threshold < 0:
            raise ValueError("threshold must be non-negative.")
        self.epsilon = epsilon
        self.max_iter = int(max_iter)
        self.threshold = threshold
        self.check_every = int(check_every)

    def _prepare(self, x, y, x_sizes, y_sizes, x_weights, y_weights):
        if not (x.is_cuda and y.is_cuda):
            raise ValueError("point clouds must be CUDA tensors")
        if x.dim() != 2 or y.dim() != 2 or x.shape[1] != 3 or y.shape[1] != 3:
            raise ValueError("x and y must be (N, 3) packed point clouds")
        nx, ny = [int(k) for k in x_sizes], [int(k) for k in y_sizes]
        if len(nx) != len(ny) or len(nx) == 0:
            raise ValueError("x_sizes and y_sizes must list the same number (>= 1) of problems")
        if sum(nx) != x.shape[0] or sum(ny) != y.shape[0] or min(nx) < 1 or min(ny) < 1:
            raise ValueError("cloud sizes must be positive and sum to the packed lengths")
        la = _log_weights(x_weights, nx, x)
        lb = _log_weights(y_weights, ny, y)
        return nx, ny, la, lb

    def __call__(self, x, y, x_sizes, y_sizes, x_weights=None, y_weights=None) -> Tensor:
        nx, ny, la, lb = self._prepare(x, y, x_sizes, y_sizes, x_weights, y_weights)
        cost, _, _, _ = _PointCloudCost.apply(x, y, la, lb, nx, ny, self.epsilon, self.max_iter,
                                              self.threshold, self.check_every)
        return cost

    @torch.no_grad()
    def solve(self, x, y, x_sizes, y_sizes, x_weights=None, y_weights=None) -> dict:
        nx, ny, la, lb = self._prepare(x, y, x_sizes, y_sizes, x_weights, y_weights)
        f, g, cost, its = _solve(x.contiguous().float(), y.contiguous().float(), la, lb, nx, ny,
                                 self.epsilon, self.max_iter, self.threshold, self.check_every)
        return {"cost": cost, "f": f, "g": g, "iterations": its}
