"""Host-side behaviour that needs no GPU: argument validation, structuring
elements, sampling normalisation, the CPU Sinkhorn path and the multi-rank
helpers (gloo, world size 2)."""

import os

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp
from scipy import ndimage as ndi

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import distance_transform as dtm
from torchmorph_gb300.distributed import max_over_ranks, split_batch

CPU = torch.zeros((1, 1, 4, 4))

ALL_OPS = [tm.grey_erosion, tm.grey_dilation, tm.grey_opening, tm.grey_closing,
           tm.morphological_gradient, tm.morphological_laplace, tm.white_tophat, tm.black_tophat]


@pytest.mark.parametrize("op", ALL_OPS)
def test_grey_requires_cuda(op):
    with pytest.raises(ValueError, match="CUDA"):
        op(CPU, size=3)


@pytest.mark.parametrize("op", [tm.binary_erosion, tm.binary_dilation, tm.binary_opening,
                                tm.binary_closing, tm.binary_propagation, tm.binary_fill_holes,
                                tm.binary_hit_or_miss])
def test_binary_requires_cuda(op):
    with pytest.raises(ValueError, match="CUDA"):
        op(CPU)


@pytest.mark.parametrize("op", [tm.euclidean_distance_transform, tm.chamfer_distance_transform,
                                tm.brute_force_distance_transform])
def test_distance_requires_cuda(op):
    with pytest.raises(ValueError, match="CUDA"):
        op(torch.zeros((1, 1, 3)))


@pytest.mark.parametrize("rank,conn", [(1, 1), (2, 1), (2, 2), (3, 1), (3, 2), (3, 3), (4, 4)])
def test_generate_binary_structure(rank, conn):
    np.testing.assert_array_equal(tm.generate_binary_structure(rank, conn).numpy(),
                                  ndi.generate_binary_structure(rank, conn))


@pytest.mark.parametrize("it", [1, 2, 3])
def test_iterate_structure(it):
    for st in [ndi.generate_binary_structure(2, 1), ndi.generate_binary_structure(3, 2),
               np.array([[0, 1, 1], [1, 0, 0], [0, 0, 1]], bool)]:
        got = tm.iterate_structure(torch.as_tensor(st), it)
        np.testing.assert_array_equal(got.numpy(), ndi.iterate_structure(st, it))
    got, origin = tm.iterate_structure(torch.as_tensor(st), it, origin=(1, -1))
    assert origin == [it, -it]


def test_structure_errors():
    with pytest.raises(ValueError, match="connectivity"):
        tm.generate_binary_structure(2, 3)


def test_sampling_normalisation():
    assert dtm._normalize_sampling(None, 3) == [1.0, 1.0, 1.0]
    assert dtm._normalize_sampling(0.5, 2) == [0.5, 0.5]
    assert dtm._normalize_sampling([0.5], 2) == [0.5, 0.5]
    for bad in ([1.0, 2.0, 3.0], 0.0, -1.0, float("inf"), float("nan")):
        with pytest.raises(ValueError, match="sampling"):
            dtm._normalize_sampling(bad, 2)


def test_sinkhorn_cpu_path_matches_oracle():
    g = torch.Generator().manual_seed(41)
    src = torch.rand((2, 8), generator=g, dtype=torch.float64) + 0.1
    tgt = torch.rand((2, 8), generator=g, dtype=torch.float64) + 0.1
    for log_space in (False, True):
        solver = tm.SinkhornSolver(epsilon=1.5, max_iter=500, log_space=log_space)
        a, b, c = solver.data_preprocess(src, tgt)
        lu, lv, _ = oracle.sinkhorn(a.numpy(), b.numpy(), c.numpy(), 1.5, 500, log_space=log_space)
        dist, _, _ = oracle.sinkhorn_cost(c.numpy(), lu, lv, 1.5)
        np.testing.assert_allclose(solver(src, tgt).numpy(), dist, rtol=1e-10)


def test_sinkhorn_one_solve_per_problem(monkeypatch):
    """forward, plan, potentials and solve on the same (unmodified) inputs run one solve;
    changed inputs, in-place edits or parameters solve again; results equal a fresh
    solver's, gradients still reach the inputs."""
    import torchmorph_gb300.optimal_transport as ot

    calls = []
    real = ot._torch_iterations

    def counting(*args, **kw):
        calls.append(1)
        return real(*args, **kw)

    monkeypatch.setattr(ot, "_torch_iterations", counting)
    g = torch.Generator().manual_seed(43)
    src = (torch.rand((3, 6), generator=g, dtype=torch.float64) + 0.1).requires_grad_(True)
    tgt = torch.rand((3, 6), generator=g, dtype=torch.float64) + 0.1
    solver = tm.SinkhornSolver(epsilon=1.5, max_iter=200)
    dist = solver(src, tgt)
    plan = solver.plan(src, tgt)
    f, h = solver.potentials(src, tgt)
    res = solver.solve(src, tgt)
    assert len(calls) == 1
    fresh = tm.SinkhornSolver(epsilon=1.5, max_iter=200)
    assert torch.equal(plan, fresh.plan(src, tgt))
    assert torch.equal(f, fresh.potentials(src, tgt)[0]) and torch.equal(dist.detach(), res["distance"])
    dist.sum().backward()
    assert src.grad is not None and torch.isfinite(src.grad).all()
    n = len(calls)
    with torch.no_grad():
        tgt.mul_(1.0)  # an in-place edit bumps the version counter
    solver.plan(src, tgt)
    assert len(calls) == n + 1
    solver.plan(src, tgt.clone())  # another tensor object
    assert len(calls) == n + 2
    solver.epsilon = 2.0
    solver.plan(src, tgt)
    assert len(calls) == n + 3
    every = tm.SinkhornSolver(epsilon=1.5, max_iter=200, reuse_solves=False)
    every.plan(src, tgt)
    every.plan(src, tgt)
    assert len(calls) == n + 5


@pytest.mark.parametrize("log_space", [True, False])
def test_sinkhorn_cost_gradient_is_the_envelope_gradient(log_space):
    """d/dC of sum_b w_b <P_b, C> through the solver = sum_b w_b P_b, and that is the
    derivative of the regularised cost W_b(C) = <a, f> + <b, g> - eps sum_ij P_ij
    (f = eps log u, g = eps log v at the optimum): central differences of W along a
    random direction, float64."""
    import torchmorph_gb300.optimal_transport as ot

    g = torch.Generator().manual_seed(5)
    n, d, eps = 3, 7, 0.5
    src = torch.rand((n, d), generator=g, dtype=torch.float64) + 0.1
    tgt = torch.rand((n, d), generator=g, dtype=torch.float64) + 0.1
    C = torch.rand((d, d), generator=g, dtype=torch.float64)
    w = torch.rand(n, generator=g, dtype=torch.float64)
    solver = tm.SinkhornSolver(epsilon=eps, max_iter=20000, threshold=1e-15, log_space=log_space)
    Cg = C.clone().requires_grad_(True)
    (solver(src, tgt, Cg) * w).sum().backward()
    P = solver.plan(src, tgt, C)
    torch.testing.assert_close(Cg.grad, (w[:, None, None] * P).sum(0), rtol=1e-12, atol=1e-15)

    def regularised(Cx):
        a, b, c = solver.data_preprocess(src, tgt, Cx)
        lu, lv = ot._torch_iterations(a, b, c, eps, 20000, 1e-15, True)
        mass = torch.exp(lu[:, :, None] + lv[:, None, :] - c / eps).sum((-2, -1))
        return ((a * eps * lu).sum(-1) + (b * eps * lv).sum(-1) - eps * mass) @ w

    delta = torch.rand((d, d), generator=g, dtype=torch.float64) - 0.5
    h = 1e-5
    fd = (regularised(C + h * delta) - regularised(C - h * delta)) / (2 * h)
    torch.testing.assert_close(fd, (Cg.grad * delta).sum(), rtol=1e-7, atol=1e-10)


def test_sinkhorn_argument_errors():
    with pytest.raises(ValueError, match="epsilon"):
        tm.SinkhornSolver(epsilon=0)
    with pytest.raises(ValueError, match="max_iter"):
        tm.SinkhornSolver(max_iter=0)
    s = tm.SinkhornSolver(epsilon=1.5, max_iter=10)
    with pytest.raises(ValueError, match=r"\(n, d\)"):
        s(torch.rand(4), torch.rand(4))
    with pytest.raises(ValueError, match="cost_matrix"):
        s(torch.rand(2, 4), torch.rand(2, 4), cost_matrix=torch.zeros(3, 3))


def test_split_batch():
    for n in (0, 1, 7, 256):
        for w in (1, 2, 3, 8):
            parts = [split_batch(n, r, w) for r in range(w)]
            sizes = [p.stop - p.start for p in parts]
            assert sum(sizes) == n and max(sizes) - min(sizes) <= 1
            assert all(parts[i].stop == parts[i + 1].start for i in range(w - 1))


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    x = np.random.default_rng(0).random((4, 1, 12, 11, 10)) < 0.9
    mine = x[split_batch(4, rank, world)]
    _, d, _ = oracle.edt(mine)
    out[rank] = (float(d.sum()), max_over_ranks(float(rank) + 0.5))
    torch.distributed.destroy_process_group()


def test_two_rank_batch_split_gloo():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    x = np.random.default_rng(0).random((4, 1, 12, 11, 10)) < 0.9
    _, d, _ = oracle.edt(x)
    assert abs(out[0][0] + out[1][0] - float(d.sum())) < 1e-6
    assert out[0][1] == out[1][1] == 1.5
