"""Entropic optimal transport (reference torchmorph/optimal_transport.py).

``SinkhornSolver`` keeps the reference's constructor, forward / plan /
potentials API, preprocessing and autograd contract.  CUDA float32 inputs are
solved by libtmcore in one call each, with no host synchronisation:

* many histogram pairs sharing one cost (``tensor_cores=None`` picks this
  for n >= 32 pairs of d >= 256 points; ``True`` forces it) run the
  tensor-core solver ``_C.sinkhorn_tc_solve``: the K v and K^T u products of
  all pairs as one error-compensated BF16 GEMM per half-iteration and the
  transport cost as one more GEMM;
* otherwise the FP32 solver ``_C.sinkhorn_f32_solve``: the reference's
  scaling or log-domain iterations as tiled CUDA-core contractions, every
  iteration of the solve in one persistent launch, the transport cost
  <P, C> fused (no (n, d, d) plan is materialised).

With ``threshold > 0`` both stop once every pair's L1 row-marginal residual
is <= threshold (checked every 10 iterations).  Inputs that are not CUDA
float32 tensors (CPU tensors, float64) run the reference's torch iterations
(:func:`_torch_iterations`), so the module stays a drop-in for them.

Gradients (envelope theorem): w.r.t. the histograms, the centred dual
potentials (the reference's rule); w.r.t. the cost matrix, sum_b g_b P_b,
computed by ``_C.sinkhorn_cost_grad`` from the potentials without storing a
plan (the reference returns no cost gradient).
"""

from __future__ import annotations

import weakref
from typing import NamedTuple, Optional

import torch
from torch import Tensor, nn


def build_cost_matrix(shape, p=2, device=None) -> Tensor:
    """(d, d) pairwise L^p distances between the d points of a grid of `shape`."""
    grids = torch.meshgrid([torch.arange(s, device=device) for s in shape], indexing="ij")
    pts = torch.stack(grids, dim=-1).reshape(-1, len(shape)).float()
    return torch.cdist(pts, pts, p=p)


_TC_MIN_PAIRS = 32
_TC_MIN_POINTS = 256
_CHECK_EVERY = 10


class _Solution(NamedTuple):
    log_u: Tensor          # (n, d) log-potentials (the reference's u.log() / log_u)
    log_v: Tensor
    cost: Optional[Tensor]     # (n,) <P, C> in float64 when the solver computed it
    row_err: Optional[Tensor]  # (n,) L1 row-marginal residual of the returned potentials
    iterations: object         # int, or a 0-dim device tensor (read only by solve())


def _on_device(t: Tensor) -> bool:
    return t.is_cuda and t.dtype == torch.float32


def _use_tensor_cores(a: Tensor, cost_matrix: Tensor, tensor_cores) -> bool:
    eligible = _on_device(a) and cost_matrix.shape == (a.shape[1], a.shape[1])
    if tensor_cores is None:
        return eligible and a.shape[0] >= _TC_MIN_PAIRS and a.shape[1] >= _TC_MIN_POINTS
    if tensor_cores and not eligible:
        raise ValueError("tensor_cores=True needs CUDA float32 histograms and a (d, d) cost.")
    return bool(tensor_cores)


# Largest d for which build_cost_matrix((d,), p=2) is exactly |i - j| in float32 (its
# matrix-product evaluation keeps i^2 + j^2 below 2^24); p = 1 is exact for every d.
_LINE_EXACT_P2 = 2896


def _line_cost_ok(a: Tensor, p, tensor_cores) -> bool:
    """The FP32 device solver takes the default cost (points 0 .. d-1 on a line) without a
    matrix when it equals build_cost_matrix((d,), p) bit for bit."""
    d = a.shape[1]
    if not _on_device(a) or p not in (1, 2) or (p == 2 and d > _LINE_EXACT_P2):
        return False
    eye = torch.empty((d, d), device="meta")  # shape only: the tensor-core choice needs no values
    return not _use_tensor_cores(a, eye, tensor_cores)


def _device_solve(a, b, cost_matrix, epsilon, max_iter, threshold, log_space, tensor_cores):
    """One libtmcore call: the whole solve, its transport cost and residual."""
    from . import _C

    a, b = a.contiguous(), b.contiguous()
    if tensor_cores:
        out = _C.sinkhorn_tc_solve(a, b, cost_matrix, epsilon, max_iter, threshold, _CHECK_EVERY)
    else:
        out = _C.sinkhorn_f32_solve(a, b, cost_matrix, epsilon, max_iter, threshold, log_space,
                                    _CHECK_EVERY)
    return _Solution(*out)


def _torch_iterations(a, b, cost_matrix, epsilon, max_iter, threshold, log_space):
    """The reference's iterations for inputs that are not CUDA float32 (its CPU /
    float64 path, optimal_transport.py:84-93 and 115-125): u is updated first,
    scaling denominators carry +1e-12, and with threshold > 0 the loop stops
    when, at an iteration i with i % 10 == 0, the largest L1 change of u over
    the pairs is <= threshold.  Returns the log-potentials."""
    if log_space:
        log_k = -cost_matrix / epsilon
        num = (a.log(), b.log())
        mats = (log_k, log_k.mT)
        state = [torch.zeros_like(a), torch.zeros_like(b)]

        def half(k, other):
            return num[k] - torch.logsumexp(mats[k] + other.unsqueeze(-2), dim=-1)
    else:
        kern = torch.exp(-cost_matrix / epsilon)
        num = (a, b)
        mats = (kern.mT, kern)
        state = [torch.ones_like(a), torch.ones_like(b)]

        def half(k, other):
            return num[k] / (other @ mats[k] + 1e-12)

    for i in range(max_iter):
        before = state[0]
        state[0] = half(0, state[1])
        state[1] = half(1, state[0])
        if threshold > 0 and i % 10 == 0 and (state[0] - before).abs().sum(dim=-1).max() <= threshold:
            break
    if log_space:
        return state[0], state[1]
    return state[0].log(), state[1].log()


def _plan(log_u, log_v, cost_matrix, epsilon):
    """(n, d, d) plans exp((log u - C / eps) + log v) with the reference's rounding."""
    if _on_device(log_u):
        from . import _C

        return _C.sinkhorn_plan(log_u.contiguous(), log_v.contiguous(), cost_matrix, epsilon)
    plan = torch.sub(log_u.unsqueeze(-1), (cost_matrix / epsilon).unsqueeze(0))
    plan.add_(log_v.unsqueeze(-2))
    return plan.exp_()


class _SinkhornDistance(torch.autograd.Function):
    """<P, C> of a solve, with envelope-theorem gradients: the centred dual
    potentials for a and b, sum_b g_b P_b for the cost matrix."""

    @staticmethod
    def forward(ctx, a, b, cost_matrix, epsilon, log_u, log_v, cost):
        if cost is not None:  # computed by the device solver
            distance = cost.to(a.dtype)
        else:
            distance = (_plan(log_u, log_v, cost_matrix, epsilon) * cost_matrix).sum(dim=(-2, -1))
        f = epsilon * log_u
        g = epsilon * log_v
        ctx.epsilon = epsilon
        ctx.save_for_backward(f - f.mean(dim=-1, keepdim=True), g - g.mean(dim=-1, keepdim=True),
                              log_u, log_v, cost_matrix)
        return distance

    @staticmethod
    def backward(ctx, grad_output):
        f, g, log_u, log_v, cost_matrix = ctx.saved_tensors
        grad = grad_output.unsqueeze(-1)
        grad_cost = None
        if ctx.needs_input_grad[2]:
            if _on_device(log_u):
                from . import _C

                grad_cost = _C.sinkhorn_cost_grad(log_u.contiguous(), log_v.contiguous(), cost_matrix,
                                                  ctx.epsilon, grad_output.float().contiguous())
            else:
                plan = _plan(log_u, log_v, cost_matrix, ctx.epsilon)
                grad_cost = (grad_output.to(plan.dtype)[:, None, None] * plan).sum(0)
        return grad * f, grad * g, grad_cost, None, None, None, None


class SinkhornSolver(nn.Module):
    """Entropy-regularised balanced OT between (n, d) histogram batches sharing a (d, d) cost."""

    def __init__(self, epsilon=1.0, max_iter=100, threshold=0.0, p=2, log_space=False,
                 tensor_cores=None, reuse_solves=True):
        super().__init__()
        if epsilon <= 0:
            raise ValueError("epsilon must be positive.")
        if max_iter <= 0:
            raise ValueError("max_iter must be positive.")
        if threshold < 0:
            raise ValueError("threshold must be non-negative.")
        self.epsilon = epsilon
        self.max_iter = max_iter
        self.threshold = threshold
        self.p = p
        self.log_space = log_space
        self.tensor_cores = tensor_cores
        # the last solve (see _solve), reused by forward / plan / potentials / solve on the
        # same problem unless reuse_solves is False (then every call solves)
        self.reuse_solves = reuse_solves
        self._last = None

    def extra_repr(self):
        return (
            f"epsilon={self.epsilon}, max_iter={self.max_iter}, "
            f"threshold={self.threshold}, log_space={self.log_space}"
        )

    def data_preprocess(self, source, target, cost_matrix: Optional[Tensor] = None):
        """Validate (n, d) inputs, clamp negatives and normalise each row to unit mass."""
        return self._preprocess(source, target, cost_matrix, build=True)

    def _preprocess(self, source, target, cost_matrix, build):
        """data_preprocess; with build=False and no cost_matrix, the returned cost is None
        when the device solver computes the default line cost itself."""
        if source.ndim != 2 or source.shape != target.shape:
            raise ValueError("source and target must be (n, d) tensors of the same shape.")
        if not source.is_floating_point():
            raise ValueError("source and target must be floating-point tensors.")
        d = source.shape[1]
        if cost_matrix is None and not build and _line_cost_ok(source, self.p, self.tensor_cores):
            pass
        elif cost_matrix is None:
            cost_matrix = build_cost_matrix((d,), self.p, source.device)
        elif cost_matrix.shape != (d, d):
            raise ValueError(
                f"cost_matrix must have shape ({d}, {d}), got {tuple(cost_matrix.shape)}."
            )
        if cost_matrix is not None:
            cost_matrix = cost_matrix.to(device=source.device, dtype=source.dtype).contiguous()
        source = source.clamp(min=0)
        target = target.clamp(min=0)
        source = source / source.sum(dim=-1, keepdim=True).clamp(min=1e-12)
        target = target / target.sum(dim=-1, keepdim=True).clamp(min=1e-12)
        return source, target, cost_matrix

    def _solve(self, inputs, a, b, cost_matrix) -> _Solution:
        """The solution of the preprocessed problem (a, b, cost_matrix).  The last
        solve is kept and returned again while the caller's tensors `inputs` (source,
        target, cost or None) are the same objects, unmodified (version counters),
        and the solver's parameters are unchanged: forward, plan, potentials and solve
        on one problem run one solve.  The solver holds weak references only, so it
        keeps no input alive.  Edits made through ``.data`` do not move the version
        counter: a caller that mutates its inputs that way constructs the solver with
        ``reuse_solves=False``."""
        params = (self.epsilon, self.max_iter, self.threshold, self.log_space, self.tensor_cores, self.p)
        versions = tuple(None if t is None else t._version for t in inputs)
        last = self._last
        if self.reuse_solves and last is not None and last[0] == params and last[2] == versions and all(
                (r is None and t is None) or (r is not None and r() is t) for r, t in zip(last[1], inputs)):
            return last[3]
        with torch.no_grad():
            a, b = a.detach(), b.detach()
            c = None if cost_matrix is None else cost_matrix.detach()
            if _on_device(a):
                result = _device_solve(a, b, c, self.epsilon, self.max_iter, self.threshold, self.log_space,
                                       c is not None and _use_tensor_cores(a, c, self.tensor_cores))
            else:
                if self.tensor_cores:
                    _use_tensor_cores(a, c, True)  # raises: tensor cores need CUDA float32
                log_u, log_v = _torch_iterations(a, b, c, self.epsilon, self.max_iter, self.threshold,
                                                 self.log_space)
                result = _Solution(log_u, log_v, None, None, self.max_iter)
        refs = tuple(None if t is None else weakref.ref(t) for t in inputs)
        self._last = (params, refs, versions, result)
        return result

    def forward(self, source: Tensor, target: Tensor, cost_matrix: Optional[Tensor] = None):
        """(n,) transport distances <P, C> between the rows of source and target."""
        inputs = (source, target, cost_matrix)
        a, b, c = self._preprocess(source, target, cost_matrix, build=False)
        sol = self._solve(inputs, a, b, c)
        return _SinkhornDistance.apply(a, b, c, self.epsilon, sol.log_u, sol.log_v, sol.cost)

    @torch.no_grad()
    def solve(self, source: Tensor, target: Tensor, cost_matrix: Optional[Tensor] = None):
        """One solve with its diagnostics: a dict with ``distance`` (n,), centred
        potentials ``f``, ``g`` (n, d), ``marginal_error`` (n,) -- the L1 distance
        between the plan's row sums and the source histogram, in float64 -- and
        ``iterations`` (an int; reading it synchronises with the device)."""
        inputs = (source, target, cost_matrix)
        source, target, cost_matrix = self._preprocess(source, target, cost_matrix, build=False)
        sol = self._solve(inputs, source, target, cost_matrix)
        if sol.cost is not None:
            distance, row_err = sol.cost.to(source.dtype), sol.row_err
        else:
            plan = _plan(sol.log_u, sol.log_v, cost_matrix, self.epsilon)
            distance = (plan * cost_matrix).sum(dim=(-2, -1))
            row_err = (plan.double().sum(-1) - source.double()).abs().sum(-1)
        f = self.epsilon * sol.log_u
        g = self.epsilon * sol.log_v
        return {"distance": distance, "f": f - f.mean(dim=-1, keepdim=True),
                "g": g - g.mean(dim=-1, keepdim=True), "marginal_error": row_err,
                "iterations": int(sol.iterations)}

    @torch.no_grad()
    def plan(self, source: Tensor, target: Tensor, cost_matrix: Optional[Tensor] = None):
        """(n, d, d) transport plans exp((log u - C / eps) + log v), with the
        reference's operations and rounding; CUDA float32 plans are written by one
        kernel pass."""
        inputs = (source, target, cost_matrix)
        source, target, cost_matrix = self._preprocess(source, target, cost_matrix, build=False)
        sol = self._solve(inputs, source, target, cost_matrix)
        return _plan(sol.log_u, sol.log_v, cost_matrix, self.epsilon)

    @torch.no_grad()
    def potentials(self, source: Tensor, target: Tensor, cost_matrix: Optional[Tensor] = None):
        """Centred dual potentials (f, g), each (n, d)."""
        inputs = (source, target, cost_matrix)
        source, target, cost_matrix = self._preprocess(source, target, cost_matrix, build=False)
        sol = self._solve(inputs, source, target, cost_matrix)
        f = self.epsilon * sol.log_u
        g = self.epsilon * sol.log_v
        return f - f.mean(dim=-1, keepdim=True), g - g.mean(dim=-1, keepdim=True)
