"""Distance-transform parity: EDT / chamfer / brute force vs the oracle and scipy.

Unit spacing is bit-exact (distances, squared distances and feature indices).
Sampled EDT distances are compared to within 1 ulp of float32(scipy);
their indices with the tie-agnostic property check.
"""

import numpy as np
import pytest
import torch
from scipy import ndimage as ndi

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import _C
from tests.helpers import per_item, per_item_indices, rng

pytestmark = pytest.mark.gpu


def _t(x, dtype=None):
    return torch.as_tensor(np.ascontiguousarray(x), dtype=dtype, device="cuda")


def lattice(shape):
    v = np.ones(shape, np.float32)
    v[(slice(None), slice(None), *[slice(None, None, 2)] * (len(shape) - 2))] = 0
    return v


EDT_SHAPES = [
    ((4, 1, 128, 128, 128), 0.9),   # the 3-D exact EDT workload
    ((3, 2, 17, 19, 13), 0.9),
    ((2, 1, 64, 200), 0.97),
    ((2, 1, 1000, 3), 0.99),        # long axis-0 lines
    ((1, 1, 5, 900), 0.999),        # long last-axis lines: workspace stack
    ((2, 1, 300), 0.8),
    ((1, 2, 6, 5, 4, 3), 0.7),
    ((1, 1, 2, 3, 2, 3, 2, 2, 3, 2), 0.6),
    ((2, 1, 40, 40), 1.0),          # all foreground
    ((2, 1, 40, 41), -1.0),         # all background
]


@pytest.mark.parametrize("shape,p", EDT_SHAPES)
@pytest.mark.parametrize("dtype", [torch.bool, torch.float32])
def test_edt_exact_vs_oracle(cuda, shape, p, dtype):
    x = rng(len(shape) * 7 + shape[-1]).random(shape) < p
    d, idx = tm.euclidean_distance_transform(_t(x, dtype), return_indices=True)
    sq, od, oi = oracle.edt(x)
    np.testing.assert_array_equal(d.cpu().numpy(), od.astype(np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    s = tm.euclidean_distance_transform_squared(_t(x, dtype))
    np.testing.assert_array_equal(s.cpu().numpy(), sq.astype(np.int32))


def test_edt_single_seed_and_scipy(cuda):
    x = np.ones((1, 1, 64, 65, 33), bool)
    x[0, 0, 5, 60, 2] = False
    d, idx = tm.euclidean_distance_transform(_t(x), return_indices=True)
    ed, ei = per_item_indices(x, ndi.distance_transform_edt)
    np.testing.assert_array_equal(d.cpu().numpy(), ed.astype(np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy(), ei)


@pytest.mark.parametrize("nd", [1, 2, 3])
def test_edt_reference_lattice_cases(cuda, nd):
    shape = {1: (2, 1, 7), 2: (2, 1, 5, 6), 3: (1, 2, 4, 5, 6)}[nd]
    x = lattice(shape)
    d, idx = tm.euclidean_distance_transform(_t(x), return_indices=True)
    ed, ei = per_item_indices(x, ndi.distance_transform_edt)
    np.testing.assert_array_equal(d.cpu().numpy(), ed.astype(np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy(), ei)


def _ulps(a, b):
    a = a.astype(np.float32).view(np.int32).astype(np.int64)
    b = b.astype(np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


@pytest.mark.parametrize("shape,samp", [((2, 1, 48, 40, 36), (1.0, 1.0, 2.5)),
                                        ((2, 1, 60, 70), (0.5, 2.0)),
                                        ((2, 2, 3, 3, 3, 3), (0.5, 1.5, 2.5, 3.5))])
def test_edt_sampled_within_one_ulp(cuda, shape, samp):
    x = rng(5).random(shape) < 0.85
    d, idx = tm.euclidean_distance_transform(_t(x), sampling=samp, return_indices=True)
    ed = per_item(x, ndi.distance_transform_edt, sampling=samp)
    assert _ulps(d.cpu().numpy(), ed).max() <= 1
    # indices describe the distances (tie-agnostic, as the reference's tests check)
    idx = idx.cpu().numpy().astype(np.int64)
    grid = np.indices(shape[2:])
    for b in range(shape[0]):
        for c in range(shape[1]):
            ii = idx[:, b, c]
            assert np.all(x[b, c][tuple(ii)] == 0)
            rec = np.sqrt(sum(((g - i) * s) ** 2 for g, i, s in zip(grid, ii, samp)))
            assert _ulps(rec, ed[b, c]).max() <= 1


def test_edt_all_foreground_sampling(cuda):
    for nd in (1, 2, 4):
        x = np.ones((2, 2) + (3,) * nd, np.float32)
        samp = [0.5 + k for k in range(nd)]
        d, idx = tm.euclidean_distance_transform(_t(x), sampling=samp, return_indices=True)
        ed, ei = per_item_indices(x, ndi.distance_transform_edt, sampling=samp)
        np.testing.assert_array_equal(d.cpu().numpy(), ed.astype(np.float32))
        np.testing.assert_array_equal(idx.cpu().numpy(), ei)


@pytest.mark.parametrize("metric", ["chessboard", "taxicab", "chamfer345"])
@pytest.mark.parametrize("shape,p", [((2, 1, 64, 64, 64), 0.9), ((3, 1, 40, 57), 0.95),
                                     ((2, 1, 200), 0.9), ((1, 2, 5, 6, 7, 4), 0.8),
                                     ((1, 1, 30, 30), 1.0), ((1, 1, 20, 40), 0.995)])
def test_cdt_exact_vs_oracle(cuda, metric, shape, p):
    if metric == "chamfer345" and len(shape) > 5:
        pytest.skip("3-4-5 chamfer is defined for up to 3 spatial dims")
    x = rng(len(shape) + shape[-1]).random(shape) < p
    d, idx = tm.chamfer_distance_transform(_t(x), metric=metric, return_indices=True)
    od, oi = oracle.cdt(x, metric)
    exp = np.where(od < 0, -1.0, od.astype(np.float32) / (3.0 if metric == "chamfer345" else 1.0))
    np.testing.assert_array_equal(d.cpu().numpy(), exp.astype(np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    if metric != "chamfer345":
        sd, si = per_item_indices(x, ndi.distance_transform_cdt, metric=metric)
        np.testing.assert_array_equal(d.cpu().numpy(), sd.astype(np.float32))
        np.testing.assert_array_equal(idx.cpu().numpy(), si)


@pytest.mark.parametrize("metric", ["euclidean", "taxicab", "chessboard"])
@pytest.mark.parametrize("shape,p", [((2, 1, 23, 31), 0.8), ((1, 2, 9, 8, 7), 0.9),
                                     ((2, 1, 50), 0.7), ((1, 1, 6, 6), 1.0), ((1, 1, 6, 6), -1.0)])
def test_bfdt_vs_oracle(cuda, metric, shape, p):
    x = rng(3).random(shape) < p
    d, idx = tm.brute_force_distance_transform(_t(x), metric=metric, return_indices=True)
    od, oi = oracle.bfdt(x, metric)
    np.testing.assert_array_equal(d.cpu().numpy(), od.astype(np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)


def test_bfdt_sampled(cuda):
    x = rng(4).random((2, 1, 20, 30)) < 0.8
    d = tm.brute_force_distance_transform(_t(x), sampling=[0.5, 2.0])
    ed = per_item(x, ndi.distance_transform_bf, sampling=[0.5, 2.0])
    np.testing.assert_allclose(d.cpu().numpy(), ed, rtol=2e-7, atol=0)


@pytest.mark.parametrize("op", [tm.euclidean_distance_transform, tm.chamfer_distance_transform,
                                tm.brute_force_distance_transform])
def test_flags_outputs_and_errors(cuda, op):
    x = _t(lattice((2, 1, 5, 6)))
    d = op(x)
    i = op(x, return_distances=False, return_indices=True)
    both = op(x, return_indices=True)
    assert d.shape == x.shape and i.shape == (2, *x.shape)
    torch.testing.assert_close(both[0], d)
    torch.testing.assert_close(both[1], i)
    dist64 = torch.empty_like(x, dtype=torch.float64)
    ind = torch.empty((2, *x.shape), device="cuda", dtype=torch.int32)
    assert op(x, return_distances=False, distances=dist64, indices=ind) is None
    torch.testing.assert_close(dist64, d.double())
    torch.testing.assert_close(ind, i)
    with pytest.raises(ValueError, match="At least one"):
        op(x, return_distances=False, return_indices=False)
    with pytest.raises(ValueError, match="empty tensor"):
        op(torch.zeros((1, 1, 0), device="cuda"))
    with pytest.raises(ValueError, match="distances shape"):
        op(x, distances=torch.empty((1, 1, 2, 2), device="cuda"))
    assert not op(x.clone().requires_grad_()).requires_grad


@pytest.mark.parametrize("op", [tm.euclidean_distance_transform, tm.chamfer_distance_transform,
                                tm.brute_force_distance_transform])
def test_current_stream(cuda, op):
    inp = torch.ones((1, 1, 16, 16), device="cuda")
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        torch.cuda._sleep(5_000_000)
        inp.zero_()
        d, i = op(inp, return_indices=True)
    stream.synchronize()
    assert torch.all(d == 0)
    own = torch.stack(torch.meshgrid(torch.arange(16), torch.arange(16), indexing="ij")).to(torch.int32)
    assert torch.equal(i.cpu()[:, 0, 0], own)


def test_noncontiguous_input(cuda):
    x = np.ones((2, 2, 5, 6), np.float32)
    x[0, 0] = 0
    x[0, 1, ::2, ::2] = 0
    x[1, 0, 1::2, ::2] = 0
    x[1, 1, 2, 3] = 0
    inp = _t(x).transpose(-1, -2)
    d, i = tm.euclidean_distance_transform(inp, return_indices=True)
    ed, ei = per_item_indices(inp.cpu().numpy(), ndi.distance_transform_edt)
    np.testing.assert_array_equal(d.cpu().numpy(), ed.astype(np.float32))
    np.testing.assert_array_equal(i.cpu().numpy(), ei)


def test_edt_vector_path_and_offset_outputs(cuda):
    x = rng(11).random((2, 1, 64, 256)) < 0.95
    sq, od, oi = oracle.edt(x)
    d, i = tm.euclidean_distance_transform(_t(x), return_indices=True)
    np.testing.assert_array_equal(d.cpu().numpy(), od.astype(np.float32))
    np.testing.assert_array_equal(i.cpu().numpy(), oi)
    # outputs that start 4 bytes into their storage take the scalar store path
    dbuf = torch.empty(x.size + 1, dtype=torch.float32, device="cuda")[1:].view(x.shape)
    ibuf = torch.empty(2 * x.size + 1, dtype=torch.int32, device="cuda")[1:].view((2, *x.shape))
    tm.euclidean_distance_transform(_t(x), distances=dbuf, indices=ibuf)
    np.testing.assert_array_equal(dbuf.cpu().numpy(), od.astype(np.float32))
    np.testing.assert_array_equal(ibuf.cpu().numpy(), oi)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_edt_shell_patch_and_overflow(cuda, seed):
    """3-D items with 97..128-voxel rows take the bitmap shell search (|d|^2 <= 16); voxels
    it leaves are patched one by one, and items with more of them than the patch list
    holds (or without background) take the separable passes.  Item 0: a 9^3 foreground
    block (centre at |d|^2 = 25); item 1: a radius-12 foreground ball (~2000 listed
    voxels); item 2: all foreground (overflows the list); item 3: plain Bernoulli(0.9)."""
    r = rng(100 + seed)
    shape = (4, 1, 40, 50, 128)
    x = r.random(shape) < 0.9
    x[0, 0, 10:19, 20:29, 60:69] = True
    zz, yy, xx = np.meshgrid(np.arange(40), np.arange(50), np.arange(128), indexing="ij")
    x[1, 0] |= (zz - 20) ** 2 + (yy - 25) ** 2 + (xx - 64) ** 2 <= 144
    x[2] = True
    sq, od, oi = oracle.edt(x)
    d, idx = tm.euclidean_distance_transform(_t(x), return_indices=True)
    np.testing.assert_array_equal(d.cpu().numpy(), od.astype(np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy(), oi)
    s = tm.euclidean_distance_transform_squared(_t(x))
    np.testing.assert_array_equal(s.cpu().numpy(), sq.astype(np.int32))
    ed, ei = per_item_indices(x[[0, 1, 3]], ndi.distance_transform_edt)
    np.testing.assert_array_equal(d.cpu().numpy()[[0, 1, 3]], ed.astype(np.float32))
    np.testing.assert_array_equal(idx.cpu().numpy()[:, [0, 1, 3]], ei)


@pytest.mark.parametrize("metric", ["chessboard", "taxicab", "chamfer345"])
@pytest.mark.parametrize("variant", [-1, 2])
def test_chamfer_far_voxels(cuda, metric, variant):
    """Voxels whose nearest background lies beyond the radius-4 shell's classes are
    searched on the bitmap (the 9^3 block's centre; taxicab and 3-4-5 voxels at
    Bernoulli(0.9)); a unit with many of them (the ball, the all-foreground item) sends
    its item to the raster passes.  Fast path == raster passes == oracle, for the
    work-queue shell kernel (built-in) and the block kernel (autotuner variant 2)."""
    from torchmorph_gb300 import autotune

    r = rng(7)
    shape = (4, 1, 40, 50, 128)
    x = r.random(shape) < 0.9
    x[0, 0, 10:19, 20:29, 60:69] = True
    zz, yy, xx = np.meshgrid(np.arange(40), np.arange(50), np.arange(128), indexing="ij")
    x[1, 0] |= (zz - 20) ** 2 + (yy - 25) ** 2 + (xx - 64) ** 2 <= 144
    x[2] = True
    t = torch.from_numpy(x).cuda()
    cls = autotune.work_class("cdt_3d", t.numel())
    autotune.set_variant("cdt_3d", cls, variant)
    try:
        d_fast, _ = _C.cdt(t, metric, True, False)
    finally:
        autotune.set_variant("cdt_3d", cls, -1)
    d_ref, _ = _C.cdt(t, metric, True, True)
    np.testing.assert_array_equal(d_fast.cpu().numpy(), d_ref.cpu().numpy())
    d_o, _ = oracle.cdt(x, metric)
    if metric == "chamfer345":  # the oracle counts thirds
        d_o = np.where(d_o < 0, -1.0, d_o.astype(np.float32) / np.float32(3.0)).astype(np.float32)
    np.testing.assert_array_equal(d_fast.cpu().numpy(), d_o)


@pytest.mark.parametrize("metric", ["chessboard", "taxicab", "chamfer345"])
@pytest.mark.parametrize("shape,p", [((2, 1, 20, 33, 128), 0.9), ((1, 2, 9, 40, 100), 0.85),
                                     ((3, 1, 12, 16, 128), 0.999)])
def test_chamfer_distances_bitmap_path_vs_raster(cuda, metric, shape, p):
    """Distances-only calls on 3-D items with 97..128-voxel rows go through the bitmap
    shell search; items it cannot finish (sparse backgrounds) fall back per item.  The
    result must equal the raster passes (indices requested) and, for the scipy metrics,
    scipy itself."""
    r = rng(hash((metric, shape)) % 2**31)
    x = r.random(shape) < p
    if shape[0] == 3:
        x[1] = True          # one item without background: -1 everywhere
        x[2] = r.random(shape[2:]) < 0.9  # one dense item next to a sparse one
    t = torch.from_numpy(x).cuda()
    d_fast, _ = _C.cdt(t, metric, True, False)
    d_ref, _ = _C.cdt(t, metric, True, True)
    np.testing.assert_array_equal(d_fast.cpu().numpy(), d_ref.cpu().numpy())
    d_o, _ = oracle.cdt(x, metric)
    if metric == "chamfer345":  # the oracle counts thirds
        d_o = np.where(d_o < 0, -1.0, d_o.astype(np.float32) / np.float32(3.0)).astype(np.float32)
    np.testing.assert_array_equal(d_fast.cpu().numpy(), d_o)
    if metric != "chamfer345" and shape[0] != 3:
        exp = per_item(x, ndi.distance_transform_cdt, metric=metric).astype(np.float32)
        np.testing.assert_array_equal(d_fast.cpu().numpy(), exp)
