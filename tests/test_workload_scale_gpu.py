"""Parity at the benchmark workloads' own sizes.

The throughput figures are quoted on these inputs, so the CUDA path is checked
on exactly them, not on reduced shapes:

* the 3-D EDT volumes (4 x 128^3 bool, Bernoulli(0.9), numpy seeds 0-2):
  anisotropic sampling (1, 1, 2.5) within 1 ulp of scipy and of the oracle,
  and the chessboard, taxicab and 3-4-5 chamfer distances bit-exact against
  the oracle (and scipy for the two scipy metrics), both through the
  distances-only bitmap path the benchmark times and the raster path taken
  when indices are requested;
* the ragged batch: 256 images with H, W iid uniform in [32, 1024] (numpy
  seed 0), grey erosion 5 and 15 and binary opening of x > 0.5 through the
  persistent launches, bit-exact per image against the oracle;
* the shared-cost Sinkhorn: 256 pairs x 8192 points on the tensor cores at
  eps 0.05 and 0.01 to an L1 residual of 1e-6, with the relative OT cost
  (<= 1e-4) and the L1 row / column marginals (<= 1e-6) of 8 pairs checked
  against float64 Sinkhorn;
* the HBM-resident 8 x 4096^2 lines: binary erosion and one-pass opening
  (default cross), one-pass grey opening and white top-hat 3 x 3.
"""

import numpy as np
import pytest
import torch
from scipy import ndimage as ndi

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import RaggedBatch, SinkhornSolver, _C, ragged

pytestmark = pytest.mark.gpu

EDT_SHAPE = (4, 1, 128, 128, 128)
CROSS = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], bool)


def edt_volumes(seed):
    return np.random.default_rng(seed).random(EDT_SHAPE) < 0.9


def _ulps(a, b):
    a = a.astype(np.float32).view(np.int32).astype(np.int64)
    b = b.astype(np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


@pytest.mark.parametrize("seed", [0, 1])
def test_sampled_edt_on_the_edt_volumes(cuda, seed):
    samp = (1.0, 1.0, 2.5)
    x = edt_volumes(seed)
    d, idx = tm.euclidean_distance_transform(torch.from_numpy(x).cuda(), sampling=samp,
                                             return_indices=True)
    d = d.cpu().numpy()
    _, od, oi = oracle.edt(x, sampling=samp)
    assert _ulps(d, od).max() <= 1
    for b in range(EDT_SHAPE[0]):
        ed = ndi.distance_transform_edt(x[b, 0], sampling=samp)
        assert _ulps(d[b, 0], ed).max() <= 1
    # the indices name a nearest background voxel (ties may resolve either way in float64)
    idx = idx.cpu().numpy().astype(np.int64)
    grid = np.indices(EDT_SHAPE[2:])
    for b in range(EDT_SHAPE[0]):
        ii = idx[:, b, 0]
        assert np.all(x[b, 0][tuple(ii)] == 0)
        rec = np.sqrt(sum(((g - i) * s) ** 2 for g, i, s in zip(grid, ii, samp)))
        assert _ulps(rec, od[b, 0]).max() <= 1


@pytest.mark.parametrize("metric", ["chessboard", "taxicab", "chamfer345"])
def test_chamfer_on_the_edt_volumes(cuda, metric):
    for seed in (0, 1, 2):
        x = edt_volumes(seed)
        t = torch.from_numpy(x).cuda()
        d_fast, _ = _C.cdt(t, metric, True, False)  # the benchmarked distances-only call
        d_ras, i_ras = _C.cdt(t, metric, True, True)
        od, oi = oracle.cdt(x, metric)
        exp = np.where(od < 0, -1.0, od.astype(np.float32) / (3.0 if metric == "chamfer345" else 1.0))
        exp = exp.astype(np.float32)
        np.testing.assert_array_equal(d_fast.cpu().numpy(), exp)
        np.testing.assert_array_equal(d_ras.cpu().numpy(), exp)
        np.testing.assert_array_equal(i_ras.cpu().numpy(), oi)
        if metric != "chamfer345" and seed == 0:
            for b in range(EDT_SHAPE[0]):
                sd = ndi.distance_transform_cdt(x[b, 0], metric=metric)
                np.testing.assert_array_equal(d_fast.cpu().numpy()[b, 0], sd.astype(np.float32))


def ragged_images(seed=0, n=256):
    rng = np.random.default_rng(seed)
    shapes = [(int(rng.integers(32, 1025)), int(rng.integers(32, 1025))) for _ in range(n)]
    return [rng.random(s, dtype=np.float32) for s in shapes]


def test_ragged_workload_vs_oracle(cuda):
    imgs = ragged_images()
    rb = RaggedBatch.from_images([torch.from_numpy(im).cuda() for im in imgs])
    e5 = ragged.grey_erosion(rb, size=5)
    e15 = ragged.grey_erosion(rb, size=15)
    bo = ragged.binary_opening(rb.map(lambda v: v > 0.5))
    graph, outs = ragged.capture(
        lambda b: (ragged.grey_erosion(b, size=5), ragged.grey_erosion(b, size=15),
                   ragged.binary_opening(b.map(lambda v: v > 0.5))), rb)
    for o in outs:
        o.data.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for e, o in zip((e5, e15, bo), outs):
        assert torch.equal(e.data, o.data)
    z5, z15 = np.zeros((5, 5), np.float32), np.zeros((15, 15), np.float32)
    for k, (im, g5, g15, gb) in enumerate(zip(imgs, e5.images(), e15.images(), bo.images())):
        x = im[None, None]
        np.testing.assert_array_equal(g5.cpu().numpy(), oracle.grey(x, z5)[0, 0], err_msg=f"image {k}")
        np.testing.assert_array_equal(g15.cpu().numpy(), oracle.grey(x, z15)[0, 0], err_msg=f"image {k}")
        ob = oracle.binary(oracle.binary(x > 0.5, CROSS), CROSS, dilation=True)[0, 0]
        np.testing.assert_array_equal(gb.cpu().numpy(), ob.astype(bool), err_msg=f"image {k}")


def sinkhorn_problem(n=256, d=8192, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.rand((d, 3), generator=g, dtype=torch.float64)
    y = torch.rand((d, 3), generator=g, dtype=torch.float64)
    cost = torch.cdist(x, y).square()
    cost = (cost / cost.max()).float()
    rng = np.random.default_rng(seed)
    a = torch.tensor(rng.dirichlet(np.ones(d), n), dtype=torch.float32)
    b = torch.tensor(rng.dirichlet(np.ones(d), n), dtype=torch.float32)
    return a.cuda(), b.cuda(), cost.cuda()


@pytest.mark.parametrize("eps", [0.05, 0.01])
def test_tensor_core_sinkhorn_workload_error_bounds(cuda, eps):
    a, b, cost = sinkhorn_problem()
    solver = SinkhornSolver(epsilon=eps, max_iter=20000, threshold=1e-6, tensor_cores=True)
    res = solver.solve(a, b, cost)
    its = int(res["iterations"])
    assert its < 20000
    assert res["marginal_error"].max().item() <= 1e-6
    log_u, log_v, dist, _, _ = _C.sinkhorn_tc_solve(a, b, cost, eps, its)
    # the same iterations without the stopping test give the same distances (the
    # residual sums of the stopping test only reorder fp32 accumulations)
    torch.testing.assert_close(dist.to(torch.float32), res["distance"], rtol=2e-6, atol=0)
    # float64 Sinkhorn (scaling form) on the device for 8 pairs, run far past convergence
    pairs = 8
    K = torch.exp(-cost.double() / eps)
    A, B = a[:pairs].double(), b[:pairs].double()
    u, v = torch.ones_like(A), torch.ones_like(B)
    for _ in range(its + 2000):
        u = A / (v @ K.T)
        v = B / (u @ K)
    ref = ((u @ (K * cost.double())) * v).sum(-1)
    rel = ((dist[:pairs].double() - ref).abs() / ref).max().item()
    U, V = torch.exp(log_u[:pairs].double()), torch.exp(log_v[:pairs].double())
    rows = (U * (V @ K.T) - A).abs().sum(-1).max().item()
    cols = (V * (U @ K) - B).abs().sum(-1).max().item()
    assert rel <= 1e-4, rel
    assert rows <= 1e-6, rows
    assert cols <= 1e-6, cols


def test_hbm_resident_binary_and_grey_lines(cuda):
    """The benchmark's HBM-resident 8 x 4096^2 lines: binary erosion and the one-pass
    binary opening with the default cross (row walkers), and the one-pass grey opening and
    white top-hat 3 x 3 (register walkers + ring tiles), against the oracle on two items
    and against the two-call composition on all eight."""
    g = torch.Generator(device="cpu").manual_seed(1)
    x = torch.rand((8, 1, 4096, 4096), generator=g)
    xb = (x > 0.5).cuda()
    ero = tm.binary_erosion(xb)
    opn = tm.binary_opening(xb)
    assert torch.equal(opn, tm.binary_dilation(_C.binary_erosion_cuda(xb, torch.from_numpy(CROSS), [0, 0], False)))
    for i in (0, 7):
        xi = xb[i:i + 1].cpu().numpy()
        e = oracle.binary(xi, CROSS)
        np.testing.assert_array_equal(ero[i:i + 1].cpu().numpy(), e)
        np.testing.assert_array_equal(opn[i:i + 1].cpu().numpy(), oracle.binary(e, CROSS, dilation=True))
    xg = x.cuda()
    gop = tm.grey_opening(xg, size=3)
    assert torch.equal(gop, tm.grey_dilation(tm.grey_erosion(xg, size=3), size=3))
    assert torch.equal(tm.white_tophat(xg, size=3), xg - gop)
    z = np.zeros((3, 3), np.float32)
    xi = x[3:4].numpy()
    np.testing.assert_array_equal(gop[3:4].cpu().numpy(), oracle.grey(oracle.grey(xi, z), z, dilation=True))
