"""Shared-cost Sinkhorn on the tensor cores vs the float64 oracle and the FP32 path."""

import numpy as np
import pytest
import torch

import oracle
from torchmorph_gb300 import SinkhornSolver, _C, _lib

pytestmark = pytest.mark.gpu


def _problem(n, d, seed, zeros=False):
    """Two point clouds in [0,1]^3, squared-Euclidean cost scaled to max 1, Dirichlet(1) pairs."""
    r = np.random.default_rng(seed)
    x, y = r.random((d, 3)), r.random((d, 3))
    cost = ((x[:, None] - y[None]) ** 2).sum(-1)
    cost /= cost.max()
    a, b = r.dirichlet(np.ones(d), n), r.dirichlet(np.ones(d), n)
    if zeros:
        a[0, :7] = 0.0
        a[0] /= a[0].sum()
    f32 = lambda v: v.astype(np.float32)
    return f32(a), f32(b), f32(cost)


def _gpu(x):
    return torch.tensor(x, dtype=torch.float32, device="cuda")


def _solve(a, b, cost, eps, iters, threshold=0.0):
    out = _C.sinkhorn_tc_solve(_gpu(a), _gpu(b), _gpu(cost), eps, iters, threshold)
    torch.cuda.synchronize()
    assert _lib.load().tm_device_error(1) == 0
    log_u, log_v, dist, row_err, its = out
    return (log_u.double().cpu().numpy(), log_v.double().cpu().numpy(), dist.cpu().numpy(),
            row_err.cpu().numpy(), its)


@pytest.mark.parametrize("n,d,eps,iters", [(100, 300, 0.05, 200), (40, 256, 0.01, 150),
                                           (130, 128, 0.2, 60)])
def test_same_iterations_as_fp64_oracle(cuda, n, d, eps, iters):
    """Same start, same iteration count: the tensor-core iterates track the fp64 ones."""
    a, b, cost = _problem(n, d, seed=n + d, zeros=True)
    lu, lv, dist, row_err, its = _solve(a, b, cost, eps, iters)
    assert its == iters
    lu_o, lv_o, _ = oracle.sinkhorn(a, b, cost, eps, iters, log_space=False)
    dist_o, _, _ = oracle.sinkhorn_cost(cost, lu_o, lv_o, eps)
    # the solver's own fp64 cost and residual agree with fp64 sums over its potentials
    dist_here, rm, cm = oracle.sinkhorn_cost(cost, lu, lv, eps)
    np.testing.assert_allclose(dist, dist_here, rtol=2e-6)
    # Near convergence the residual is at the level of the products' own error
    # (~3e-7) plus the rounding of the fp32 log-potentials the fp64 sums start
    # from: exp(log u) is off by up to ulp(|log u|)/2 relative.
    floor = 4e-7 + 2.0**-24 * (np.abs(lu[np.isfinite(lu)]).max() + np.abs(lv).max())
    np.testing.assert_allclose(row_err, np.abs(rm - a).sum(-1), rtol=0, atol=floor)
    assert np.abs(cm - b).sum(-1).max() < floor  # columns are matched by the last half-step
    # and the transport cost matches the oracle's after the same iterations
    assert np.max(np.abs(dist - dist_o) / dist_o) < 1e-5
    # the plan is invariant to (u c, v / c): compare potentials centred on the valid entries
    ok = np.isfinite(lu_o)
    assert np.array_equal(np.isfinite(lu), ok)
    diff = np.where(ok, lu, 0.0) - np.where(ok, lu_o, 0.0)
    shift = diff.sum(1, keepdims=True) / ok.sum(1, keepdims=True)
    assert np.max(np.abs(np.where(ok, diff - shift, 0.0))) < 5e-4 / eps


@pytest.mark.parametrize("iters", [1, 4])
def test_residual_far_from_convergence(cuda, iters):
    a, b, cost = _problem(64, 256, seed=iters)
    lu, lv, dist, row_err, _ = _solve(a, b, cost, 0.05, iters)
    dist_here, rm, _ = oracle.sinkhorn_cost(cost, lu, lv, 0.05)
    np.testing.assert_allclose(row_err, np.abs(rm - a).sum(-1), rtol=1e-4)
    np.testing.assert_allclose(dist, dist_here, rtol=2e-6)


def test_stops_at_marginal_tolerance(cuda):
    """threshold > 0: stop once every pair's L1 row residual <= threshold (fp64 check)."""
    a, b, cost = _problem(40, 384, seed=5)
    eps, tol = 0.05, 1e-6
    lu, lv, dist, row_err, its = _solve(a, b, cost, eps, 3000, threshold=tol)
    assert its < 3000 and its % 10 == 0
    _, rm, cm = oracle.sinkhorn_cost(cost, lu, lv, eps)
    assert np.abs(rm - a).sum(-1).max() < 1.5 * tol
    assert np.abs(cm - b).sum(-1).max() < 1.5 * tol
    assert row_err.max() < 1.5 * tol
    # the converged transport cost is the fp64 solver's
    lu_o, lv_o, _ = oracle.sinkhorn(a, b, cost, eps, its + 1000, log_space=False)
    dist_o, _, _ = oracle.sinkhorn_cost(cost, lu_o, lv_o, eps)
    assert np.max(np.abs(dist - dist_o) / dist_o) < 1e-4


def test_solver_api_matches_fp32_path(cuda):
    a, b, cost = _problem(48, 256, seed=11)
    src, tgt, C = _gpu(a), _gpu(b), _gpu(cost)
    tc = SinkhornSolver(epsilon=0.05, max_iter=200, tensor_cores=True)
    fp = SinkhornSolver(epsilon=0.05, max_iter=200, log_space=True, tensor_cores=False)
    d_tc, d_fp = tc(src, tgt, C), fp(src, tgt, C)
    torch.testing.assert_close(d_tc, d_fp, rtol=1e-4, atol=0)
    f_tc, g_tc = tc.potentials(src, tgt, C)
    f_fp, g_fp = fp.potentials(src, tgt, C)
    torch.testing.assert_close(f_tc, f_fp, rtol=0, atol=2e-5)
    torch.testing.assert_close(g_tc, g_fp, rtol=0, atol=2e-5)
    torch.testing.assert_close(tc.plan(src, tgt, C), fp.plan(src, tgt, C), rtol=1e-3, atol=1e-9)
    # auto mode picks the tensor cores for >= 32 pairs of >= 256 points
    auto = SinkhornSolver(epsilon=0.05, max_iter=200)
    torch.testing.assert_close(auto(src, tgt, C), d_tc, rtol=0, atol=0)
    res = tc.solve(src, tgt, C)
    assert res["iterations"] == 200 and res["marginal_error"].dtype == torch.float64
    torch.testing.assert_close(res["distance"], d_tc, rtol=0, atol=0)


def test_backward_is_centred_potentials(cuda):
    a, b, cost = _problem(32, 256, seed=13)
    C = _gpu(cost)
    grads = []
    for flag in (True, False):
        s, t = _gpu(a).requires_grad_(), _gpu(b).requires_grad_()
        SinkhornSolver(epsilon=0.1, max_iter=100, log_space=True, tensor_cores=flag)(s, t, C).sum().backward()
        grads.append((s.grad, t.grad))
    torch.testing.assert_close(grads[0][0], grads[1][0], rtol=0, atol=1e-5)
    torch.testing.assert_close(grads[0][1], grads[1][1], rtol=0, atol=1e-5)


def test_rejects_bad_arguments(cuda):
    a = torch.full((4, 256), 1 / 256, device="cuda")
    C = torch.rand(256, 256, device="cuda")
    with pytest.raises(RuntimeError, match="epsilon"):
        _C.sinkhorn_tc_solve(a, a, C, 0.0, 10)
    with pytest.raises(RuntimeError, match="cost_matrix"):
        _C.sinkhorn_tc_solve(a, a, C[:128, :128].contiguous(), 0.1, 10)
    with pytest.raises(ValueError, match="tensor_cores"):
        SinkhornSolver(tensor_cores=True)(a.double(), a.double(), C.double())
