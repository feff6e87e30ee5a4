"""Sinkhorn parity: fused CUDA iterations vs the float64 oracle and the CPU torch path."""

import numpy as np
import pytest
import torch

import oracle
from torchmorph_gb300 import SinkhornSolver, _C, build_cost_matrix

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
