"""Ragged point-cloud Sinkhorn (one cooperative launch) vs the float64 oracle; gradients vs
float64 autograd (envelope, potentials fixed) and central finite differences."""

import numpy as np
import pytest
import torch

import oracle
from torchmorph_gb300 import PointCloudSinkhorn, _lib, pack_clouds

pytestmark = pytest.mark.gpu


def _clouds(sizes, seed):
    r = np.random.default_rng(seed)
    xs, ys = [], []
    for n, m in sizes:
        means = r.uniform(-1, 1, (4, 3))
        xs.append(means[r.integers(0, 4, n)] + 0.2 * r.standard_normal((n, 3)))
        ys.append(means[r.integers(0, 4, m)] + 0.2 * r.standard_normal((m, 3)))
    return [x.astype(np.float32) for x in xs], [y.astype(np.float32) for y in ys]


def _pack(xs, ys):
    x, nx = pack_clouds([torch.from_numpy(v).cuda() for v in xs])
    y, ny = pack_clouds([torch.from_numpy(v).cuda() for v in ys])
    return x, y, nx, ny


SIZES = [(1, 1), (3, 200), (130, 7), (257, 300), (64, 64), (500, 129), (2, 1000)]


@pytest.mark.parametrize("eps,iters", [(0.5, 30), (0.1, 60), (0.05, 100)])
def test_fixed_iterations_vs_fp64_oracle(cuda, eps, iters):
    xs, ys = _clouds(SIZES, 3)
    x, y, nx, ny = _pack(xs, ys)
    res = PointCloudSinkhorn(epsilon=eps, max_iter=iters, threshold=0.0).solve(x, y, nx, ny)
    torch.cuda.synchronize()
    assert _lib.load().tm_device_error(1) == 0
    f, g = res["f"].cpu().numpy(), res["g"].cpu().numpy()
    assert (res["iterations"].cpu().numpy() == iters).all()
    ox, oy = np.cumsum([0] + nx), np.cumsum([0] + ny)
    for p in range(len(SIZES)):
        fo, go, its, cost = oracle.pointcloud_sinkhorn(xs[p].astype(np.float64), ys[p].astype(np.float64),
                                                       eps, iters, threshold=0.0)
        assert its == iters
        # potentials are defined up to (f + c, g - c); compare the plan-invariant parts
        df = f[ox[p]:ox[p + 1]] - fo
        dg = g[oy[p]:oy[p + 1]] - go
        c = df.mean()
        assert np.abs(df - c).max() < 2e-4 and np.abs(dg + c).max() < 2e-4, (p, np.abs(df - c).max())
        np.testing.assert_allclose(res["cost"][p].item(), cost, rtol=2e-5, atol=2e-5)


def test_stops_on_marginal_threshold(cuda):
    xs, ys = _clouds([(40, 60), (100, 90), (17, 300), (256, 128)], 7)
    x, y, nx, ny = _pack(xs, ys)
    eps, tol = 0.1, 1e-4
    res = PointCloudSinkhorn(epsilon=eps, max_iter=5000, threshold=tol, check_every=10).solve(x, y, nx, ny)
    its = res["iterations"].cpu().numpy()
    f, g = res["f"].cpu().numpy(), res["g"].cpu().numpy()
    ox, oy = np.cumsum([0] + nx), np.cumsum([0] + ny)
    for p in range(4):
        _, _, its_o, cost_o = oracle.pointcloud_sinkhorn(xs[p], ys[p], eps, 5000, threshold=tol)
        assert its[p] % 10 == 0 and abs(int(its[p]) - its_o) <= 10, (its[p], its_o)
        # float64 marginals of the returned plan
        xp, yp = xs[p].astype(np.float64), ys[p].astype(np.float64)
        C = ((xp[:, None] - yp[None]) ** 2).sum(-1)
        fp, gp = f[ox[p]:ox[p + 1]].astype(np.float64), g[oy[p]:oy[p + 1]].astype(np.float64)
        P = np.exp((fp[:, None] + gp[None] - C) / eps) / (len(xp) * len(yp))
        assert np.abs(P.sum(0) - 1 / len(yp)).sum() < 3 * tol
        assert np.abs(P.sum(1) - 1 / len(xp)).sum() < 1e-4
        np.testing.assert_allclose(res["cost"][p].item(), cost_o, rtol=1e-4)


def test_gradient_vs_fp64_autograd_and_fd(cuda):
    sizes = [(30, 45), (130, 70), (9, 300)]
    xs, ys = _clouds(sizes, 11)
    x, y, nx, ny = _pack(xs, ys)
    eps = 0.1
    x.requires_grad_(True)
    y.requires_grad_(True)
    solver = PointCloudSinkhorn(epsilon=eps, max_iter=20000, threshold=1e-6)
    cost = solver(x, y, nx, ny)
    w = torch.tensor([1.0, -2.0, 0.5], device="cuda")
    (cost * w).sum().backward()
    gx, gy = x.grad.cpu().numpy(), y.grad.cpu().numpy()
    ox, oy = np.cumsum([0] + nx), np.cumsum([0] + ny)
    for p in range(len(sizes)):
        xp, yp = xs[p].astype(np.float64), ys[p].astype(np.float64)
        fo, go, _, _ = oracle.pointcloud_sinkhorn(xp, yp, eps, 100000, threshold=1e-13, check_every=1)
        # float64 autograd of the regularised dual objective with the potentials fixed
        xt = torch.tensor(xp, requires_grad=True)
        yt = torch.tensor(yp, requires_grad=True)
        C = ((xt[:, None] - yt[None]) ** 2).sum(-1)
        a, b = 1.0 / len(xp), 1.0 / len(yp)
        fo_t, go_t = torch.from_numpy(fo), torch.from_numpy(go)
        L = a * fo_t.sum() + b * go_t.sum() - eps * (a * b * (torch.exp((fo_t[:, None] + go_t[None] - C) / eps)
                                                             - 1)).sum()
        L.backward()
        np.testing.assert_allclose(gx[ox[p]:ox[p + 1]], w[p].item() * xt.grad.numpy(), rtol=2e-3, atol=2e-4)
        np.testing.assert_allclose(gy[oy[p]:oy[p + 1]], w[p].item() * yt.grad.numpy(), rtol=2e-3, atol=2e-4)
        # central finite differences of the converged float64 cost, a few coordinates
        h = 1e-3
        for (i, d) in [(0, 0), (len(xp) - 1, 2), (len(xp) // 2, 1)]:
            xpp, xpm = xp.copy(), xp.copy()
            xpp[i, d] += h
            xpm[i, d] -= h
            cp = oracle.pointcloud_sinkhorn(xpp, yp, eps, 100000, threshold=1e-13, check_every=1)[3]
            cm = oracle.pointcloud_sinkhorn(xpm, yp, eps, 100000, threshold=1e-13, check_every=1)[3]
            fd = (cp - cm) / (2 * h)
            assert abs(gx[ox[p] + i, d] - w[p].item() * fd) < 2e-3 * abs(w[p].item() * fd) + 2e-4


def test_errors(cuda):
    x = torch.rand((5, 3), device="cuda")
    with pytest.raises(ValueError, match="sum to"):
        PointCloudSinkhorn()(x, x, [2, 2], [3, 2])
    with pytest.raises(ValueError, match="same number"):
        PointCloudSinkhorn()(x, x, [5], [2, 3])
    with pytest.raises(ValueError, match="epsilon"):
        PointCloudSinkhorn(epsilon=0)
    with pytest.raises(ValueError, match="CUDA"):
        PointCloudSinkhorn()(x.cpu(), x.cpu(), [5], [5])
