"""Sinkhorn parity: fused CUDA iterations vs the float64 oracle and the CPU torch path."""

import numpy as np
import pytest
import torch

import oracle
from torchmorph_gb300 import SinkhornSolver, _C, _lib, build_cost_matrix

pytestmark = pytest.mark.gpu


def _pos(shape, seed):
    g = torch.Generator().manual_seed(seed)
    return torch.rand(shape, generator=g) + 0.1


@pytest.mark.parametrize("log_space", [False, True])
@pytest.mark.parametrize("n", [1, 3, 20])
def test_fused_matches_cpu(cuda, log_space, n):
    solver = SinkhornSolver(epsilon=1.5, max_iter=1000, log_space=log_space)
    src, tgt = _pos((n, 6), 503), _pos((n, 6), 607)
    cpu = solver(src, tgt)
    gpu = solver(src.cuda(), tgt.cuda())
    assert torch.allclose(gpu.cpu(), cpu, rtol=1e-4, atol=1e-5)
    f_c, g_c = solver.potentials(src, tgt)
    f_g, g_g = solver.potentials(src.cuda(), tgt.cuda())
    assert torch.allclose(f_g.cpu(), f_c, rtol=1e-4, atol=1e-4)
    assert torch.allclose(g_g.cpu(), g_c, rtol=1e-4, atol=1e-4)
    assert torch.allclose(solver.plan(src.cuda(), tgt.cuda()).cpu(), solver.plan(src, tgt),
                          rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("log_space", [False, True])
def test_short_run_and_backward(cuda, log_space):
    solver = SinkhornSolver(epsilon=1.5, max_iter=60, log_space=log_space)
    src, tgt = _pos((2, 6), 1409), _pos((2, 6), 1423)
    assert torch.allclose(solver(src.cuda(), tgt.cuda()).cpu(), solver(src, tgt), rtol=1e-4,
                          atol=1e-5)
    s_c, t_c = src.clone().requires_grad_(), tgt.clone().requires_grad_()
    solver(s_c, t_c).sum().backward()
    s_g, t_g = src.cuda().requires_grad_(), tgt.cuda().requires_grad_()
    solver(s_g, t_g).sum().backward()
    assert torch.allclose(s_g.grad.cpu(), s_c.grad, rtol=1e-4, atol=1e-5)
    assert torch.allclose(t_g.grad.cpu(), t_c.grad, rtol=1e-4, atol=1e-5)


@pytest.mark.parametrize("eps", [0.05, 0.5])
def test_logiter_vs_oracle(cuda, eps):
    r = np.random.default_rng(0)
    n, d = 5, 96
    pts = r.random((d, 2))
    cost = ((pts[:, None] - pts[None]) ** 2).sum(-1)
    cost /= cost.max()
    a = r.dirichlet(np.ones(d), n)
    b = r.dirichlet(np.ones(d), n)
    its = 400
    lu_o, lv_o, _ = oracle.sinkhorn(a, b, cost, eps, its, log_space=True)
    la = torch.tensor(np.log(a), dtype=torch.float32, device="cuda")
    lb = torch.tensor(np.log(b), dtype=torch.float32, device="cuda")
    M = torch.tensor(cost, dtype=torch.float32, device="cuda")
    lu = torch.zeros_like(la)
    lv = torch.zeros_like(lb)
    _C.sinkhorn_logiter(la, lb, M, M.T.contiguous(), lu, lv, its, eps)
    dist_o, _, _ = oracle.sinkhorn_cost(cost, lu_o, lv_o, eps)
    dist_g, rm, _ = oracle.sinkhorn_cost(cost, lu.double().cpu().numpy(), lv.double().cpu().numpy(),
                                         eps)
    assert np.max(np.abs(dist_g - dist_o) / dist_o) < 1e-4
    assert np.max(np.abs(rm - a).sum(-1)) < 1e-3


def test_cost_matrix_on_cuda(cuda):
    c = build_cost_matrix((3, 4), device="cuda")
    assert c.shape == (12, 12) and c.is_cuda


# ------------------------------------------------------ the FP32 device solver
def _ot_problem(n, d, seed):
    r = np.random.default_rng(seed)
    pts = r.random((d, 2))
    cost = ((pts[:, None] - pts[None]) ** 2).sum(-1)
    cost /= cost.max()
    a = r.dirichlet(np.ones(d), n)
    b = r.dirichlet(np.ones(d), n)
    return a, b, cost


def _f32(x):
    return torch.tensor(x, dtype=torch.float32, device="cuda")


def _centred(lu):
    ok = np.isfinite(lu)
    x = np.where(ok, lu, 0.0)
    return np.where(ok, x - x.sum(1, keepdims=True) / ok.sum(1, keepdims=True), 0.0)


# n = 5 and 30 take the 16-pair tiles, 70 the 64-pair tiles; d = 300 spans three
# 128-row blocks, d = 301 takes the scalar staging path (d % 4 != 0)
@pytest.mark.parametrize("log_space", [False, True])
@pytest.mark.parametrize("n,d,eps,its", [(5, 96, 0.05, 300), (30, 300, 0.1, 200), (70, 301, 0.2, 120),
                                         (1, 7, 0.5, 50)])
def test_f32_solve_vs_fp64_oracle(cuda, log_space, n, d, eps, its):
    a, b, cost = _ot_problem(n, d, seed=n + d)
    lu, lv, dist, row_err, k = _C.sinkhorn_f32_solve(_f32(a), _f32(b), _f32(cost), eps, its, 0.0, log_space)
    torch.cuda.synchronize()
    assert int(k) == its
    lu, lv = lu.double().cpu().numpy(), lv.double().cpu().numpy()
    lu_o, lv_o, _ = oracle.sinkhorn(a, b, cost, eps, its, log_space=log_space)
    # potentials up to the plan's (u c, v / c) invariance
    assert np.max(np.abs(_centred(lu) - _centred(lu_o))) < 2e-4 / eps
    # the fused cost and residual equal float64 sums over the returned potentials
    a32 = a.astype(np.float32).astype(np.float64)
    c32 = cost.astype(np.float32).astype(np.float64)
    dist_here, rm, _ = oracle.sinkhorn_cost(c32, lu, lv, eps)
    np.testing.assert_allclose(dist.cpu().numpy(), dist_here, rtol=2e-5)
    np.testing.assert_allclose(row_err.cpu().numpy(), np.abs(rm - a32).sum(-1), rtol=1e-3, atol=2e-6)
    dist_o, _, _ = oracle.sinkhorn_cost(cost, lu_o, lv_o, eps)
    assert np.max(np.abs(dist.cpu().numpy() - dist_o) / dist_o) < 1e-4


@pytest.mark.parametrize("log_space", [False, True])
def test_f32_fixed_iterations_and_early_stop(cuda, log_space):
    """The drop-in in-place iterations equal the solve's; a threshold stops on the
    device at a multiple of 10 iterations with every residual below it, and the
    stopped potentials equal a fixed run of that many iterations bit for bit."""
    n, d, eps = 40, 200, 0.1
    a, b, cost = _ot_problem(n, d, seed=3)
    A, B, C = _f32(a), _f32(b), _f32(cost)
    lu, lv, _, _, _ = _C.sinkhorn_f32_solve(A, B, C, eps, 37, 0.0, log_space)
    if log_space:
        u, v = torch.zeros_like(A), torch.zeros_like(B)
        _C.sinkhorn_logiter(A.log(), B.log(), C, C.T.contiguous(), u, v, 37, eps)
        fu, fv = u, v
    else:
        K = torch.exp(-C / eps)
        u, v = torch.ones_like(A), torch.ones_like(B)
        _C.sinkhorn_fastiter(A, B, K, K.T.contiguous(), u, v, 37)
        fu, fv = u.log(), v.log()
    torch.testing.assert_close(fu, lu, rtol=2e-6, atol=2e-6)
    torch.testing.assert_close(fv, lv, rtol=2e-6, atol=2e-6)
    tol = 1e-4
    su, sv, _, err, k = _C.sinkhorn_f32_solve(A, B, C, eps, 5000, tol, log_space)
    k = int(k)
    assert 0 < k < 5000 and k % 10 == 0
    assert err.max().item() <= 1.5 * tol
    fu2, fv2, _, _, k2 = _C.sinkhorn_f32_solve(A, B, C, eps, k, 0.0, log_space)
    assert int(k2) == k
    assert torch.equal(su, fu2) and torch.equal(sv, fv2)
    # the check before (iteration k - 10, measuring the plan after k - 11 iterations)
    # found a residual above the threshold: the solve did not stop early
    _, _, _, err_before, _ = _C.sinkhorn_f32_solve(A, B, C, eps, k - 11, 0.0, log_space)
    assert err_before.max().item() > tol * 0.9


def test_f32_solver_module_and_no_plan_in_forward(cuda):
    """SinkhornSolver on CUDA float32 below the tensor-core sizes runs the device solve;
    forward allocates no (n, d, d) plan (its peak memory stays far below one)."""
    n, d = 8, 1024
    a, b, cost = _ot_problem(n, d, seed=9)
    A, B, C = _f32(a), _f32(b), _f32(cost)
    solver = SinkhornSolver(epsilon=0.05, max_iter=100)
    solver(A, B, C)
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats()
    base = torch.cuda.memory_allocated()
    dist = SinkhornSolver(epsilon=0.05, max_iter=100)(A, B, C)
    torch.cuda.synchronize()
    # the scaling form's workspace holds K and K^T (2 d^2 floats); the plans would be n d^2
    assert torch.cuda.max_memory_allocated() - base < n * d * d * 4 // 2
    lu_o, lv_o, _ = oracle.sinkhorn(a, b, cost, 0.05, 100, log_space=False)
    dist_o, _, _ = oracle.sinkhorn_cost(cost, lu_o, lv_o, 0.05)
    assert np.max(np.abs(dist.cpu().numpy() - dist_o) / dist_o) < 1e-4


@pytest.mark.parametrize("d", [64, 130])
def test_plan_kernel_matches_the_reference_formula(cuda, d):
    n, eps = 3, 0.07
    a, b, cost = _ot_problem(n, d, seed=d)
    lu = torch.randn((n, d), device="cuda")
    lv = torch.randn((n, d), device="cuda")
    C = _f32(cost)
    got = _C.sinkhorn_plan(lu, lv, C, eps)
    ref = torch.exp(lu.unsqueeze(-1) - C / eps + lv.unsqueeze(-2))
    torch.testing.assert_close(got, ref, rtol=3e-7, atol=0)


@pytest.mark.parametrize("tensor_cores", [False, True])
def test_cost_gradient_kernel(cuda, tensor_cores):
    """grad_C = sum_b w_b P_b from the solve's potentials, against float64 torch."""
    n, d, eps = 40, 260, 0.05
    a, b, cost = _ot_problem(n, d, seed=11)
    A, B = _f32(a), _f32(b)
    C = _f32(cost).requires_grad_(True)
    w = torch.rand(n, device="cuda")
    solver = SinkhornSolver(epsilon=eps, max_iter=200, tensor_cores=tensor_cores)
    (solver(A, B, C) * w).sum().backward()
    lu, lv, _, _, _ = solver._solve((A, B, C), *solver.data_preprocess(A, B, C))
    P = torch.exp(lu.double().unsqueeze(-1) - C.detach().double() / eps + lv.double().unsqueeze(-2))
    ref = (w.double()[:, None, None] * P).sum(0)
    torch.testing.assert_close(C.grad.double(), ref, rtol=2e-5, atol=1e-9)


def test_grid_barrier_wait_budget_times_out_and_returns(cuda):
    """A poll budget of 0 makes the persistent solver's grid barriers give up: the
    device status word reports the timeout, the call returns, and with the default
    budget restored the next solve is correct again."""
    lib = _lib.load()
    n, d, eps = 70, 600, 0.1  # 5 x 2 tiles: several CTAs meet at every barrier
    a, b, cost = _ot_problem(n, d, seed=2)
    A, B, C = _f32(a), _f32(b), _f32(cost)
    ref = _C.sinkhorn_f32_solve(A, B, C, eps, 50, 0.0, False)
    torch.cuda.synchronize()
    assert lib.tm_device_error(1) == 0
    lib.tm_set_grid_wait_budget(0)
    try:
        _C.sinkhorn_f32_solve(A, B, C, eps, 50, 0.0, False)
        torch.cuda.synchronize()
        assert lib.tm_device_error(1) == 1
    finally:
        lib.tm_set_grid_wait_budget(-1)
    again = _C.sinkhorn_f32_solve(A, B, C, eps, 50, 0.0, False)
    torch.cuda.synchronize()
    assert lib.tm_device_error(1) == 0
    assert torch.equal(again[0], ref[0]) and torch.equal(again[1], ref[1])


@pytest.mark.parametrize("log_space", [False, True])
@pytest.mark.parametrize("n,d", [(3, 96), (20, 301), (5, 1500)])
def test_line_cost_equals_the_explicit_matrix(cuda, log_space, n, d):
    """With no cost matrix the FP32 solver computes |i - j| in its kernels: potentials,
    transport cost, residual, plan and histogram gradients equal, bit for bit, those of a
    solve given build_cost_matrix((d,)) -- and no (d, d) matrix is allocated."""
    a, b, _ = _ot_problem(n, d, seed=d)
    A, B = _f32(a), _f32(b)
    C = build_cost_matrix((d,), p=2, device="cuda")
    assert torch.equal(C, build_cost_matrix((d,), p=1, device="cuda"))
    eps, its = 0.1, 60
    ref = _C.sinkhorn_f32_solve(A, B, C, eps, its, 0.0, log_space)
    got = _C.sinkhorn_f32_solve(A, B, None, eps, its, 0.0, log_space)
    for r, g in zip(ref[:4], got[:4]):
        assert torch.equal(r, g)
    assert torch.equal(_C.sinkhorn_plan(ref[0], ref[1], C, eps), _C.sinkhorn_plan(got[0], got[1], None, eps))

    def module_run(cost):
        x, y = A.clone().requires_grad_(True), B.clone().requires_grad_(True)
        solver = SinkhornSolver(epsilon=eps, max_iter=its, log_space=log_space, tensor_cores=False)
        dist = solver(x, y, cost)
        dist.sum().backward()
        return dist.detach(), x.grad, y.grad, solver.plan(A, B, cost)

    for r, g in zip(module_run(C), module_run(None)):
        assert torch.equal(r, g)
    if d >= 1024:  # where one (d, d) matrix outweighs the (n, d) buffers
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        SinkhornSolver(epsilon=eps, max_iter=its, log_space=log_space, tensor_cores=False)(A, B)
        torch.cuda.synchronize()
        assert torch.cuda.max_memory_allocated() - base < d * d * 4 // 2


def test_line_cost_only_where_it_is_exact(cuda):
    from torchmorph_gb300.optimal_transport import _line_cost_ok

    A = torch.ones((2, 2896), device="cuda")
    assert _line_cost_ok(A, 2, False) and _line_cost_ok(A, 1, False)
    assert not _line_cost_ok(torch.ones((2, 2897), device="cuda"), 2, False)
    assert _line_cost_ok(torch.ones((2, 2897), device="cuda"), 1, False)
    assert not _line_cost_ok(A, 3, False)
    assert not _line_cost_ok(A.double(), 2, False)
    assert not _line_cost_ok(torch.ones((64, 512), device="cuda"), 2, None)  # tensor-core sizes
    # the matrix-product evaluation of the distances is exact up to d = 2896
    C = build_cost_matrix((2896,), p=2, device="cuda")
    i = torch.arange(2896, device="cuda", dtype=torch.float32)
    assert torch.equal(C, (i[:, None] - i[None, :]).abs())
