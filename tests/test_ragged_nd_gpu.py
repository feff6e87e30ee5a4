"""Ragged batches of 3-D volumes (one launch per operator) and the ragged EDT of 2-D
and 3-D items (one cooperative launch), bit-exact per item against the oracle."""

import numpy as np
import pytest
import torch

import oracle
from torchmorph_gb300 import RaggedBatch, ragged
from tests.helpers import rng

pytestmark = pytest.mark.gpu


def _vol_shapes(seed, n=9):
    r = rng(seed)
    shapes = [(int(r.integers(1, 24)), int(r.integers(1, 40)), int(r.integers(1, 70))) for _ in range(n)]
    return shapes + [(1, 1, 1), (3, 1, 33), (5, 9, 1), (8, 16, 64)]


def _batch(shapes, seed, binary=False):
    r = rng(seed)
    vols = [r.random(s).astype(np.float32) for s in shapes]
    if binary:
        vols = [v > 0.5 for v in vols]
    return vols, RaggedBatch.from_images([torch.from_numpy(v).cuda() for v in vols])


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("mode", ["reflect", "constant", "nearest", "mirror", "wrap"])
@pytest.mark.parametrize("size", [(3, 3, 3), (2, 5, 4), (1, 1, 7)])
def test_ragged3d_flat_grey_vs_oracle(cuda, dilation, mode, size):
    shapes = _vol_shapes(hash((dilation, mode, size)) % 1000)
    vols, rb = _batch(shapes, 1)
    r = rng(3)
    origin = tuple(int(r.integers(-(k // 2), (k - 1) // 2 + 1)) for k in size)
    op = ragged.grey_dilation if dilation else ragged.grey_erosion
    out = op(rb, size=size, mode=mode, cval=0.25, origin=origin)
    torch.cuda.synchronize()
    assert out.shapes == rb.shapes
    for v, got in zip(vols, out.images()):
        exp = oracle.grey(v[None, None], np.zeros(size, np.float32), origin=origin, mode=mode, cval=0.25,
                          dilation=dilation)[0, 0]
        np.testing.assert_array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("dilation", [False, True])
def test_ragged3d_nonflat_footprint_vs_oracle(cuda, dilation):
    vols, rb = _batch(_vol_shapes(5, n=6), 2)
    r = rng(4)
    st = r.random((3, 2, 5)).astype(np.float32)
    fp = r.random((3, 2, 5)) < 0.6
    fp[1, 1, 2] = True
    op = ragged.grey_dilation if dilation else ragged.grey_erosion
    for mode in ("reflect", "constant", "wrap"):
        out = op(rb, structure=torch.from_numpy(st), footprint=torch.from_numpy(fp), mode=mode, cval=-1.0)
        for v, got in zip(vols, out.images()):
            exp = oracle.grey(v[None, None], st, footprint=fp, mode=mode, cval=-1.0, dilation=dilation)[0, 0]
            np.testing.assert_array_equal(got.cpu().numpy(), exp)


def test_ragged3d_binary_vs_oracle(cuda):
    vols, rb = _batch(_vol_shapes(7), 3, binary=True)
    cross = np.zeros((3, 3, 3), bool)
    cross[1, 1, :] = cross[1, :, 1] = cross[:, 1, 1] = True
    box = np.ones((3, 3, 3), bool)
    for border in (False, True):
        e = ragged.binary_erosion(rb, border_value=border)  # default: the 3-D cross
        d = ragged.binary_dilation(rb, structure=torch.from_numpy(box), border_value=border)
        for v, ge, gd in zip(vols, e.images(), d.images()):
            np.testing.assert_array_equal(ge.cpu().numpy(), oracle.binary(v[None, None], cross,
                                                                          border_value=border)[0, 0].astype(bool))
            np.testing.assert_array_equal(gd.cpu().numpy(), oracle.binary(v[None, None], box, border_value=border,
                                                                          dilation=True)[0, 0].astype(bool))
    op = ragged.binary_opening(rb)
    for v, g in zip(vols, op.images()):
        exp = oracle.binary(oracle.binary(v[None, None], cross), cross, dilation=True)[0, 0]
        np.testing.assert_array_equal(g.cpu().numpy(), exp.astype(bool))


def _check_edt(items, dist_rb, idx):
    off = 0
    for v, got in zip(items, dist_rb.images()):
        _, od, oi = oracle.edt(v[None, None])
        np.testing.assert_array_equal(got.cpu().numpy(), od[0, 0].astype(np.float32))
        n = v.size
        np.testing.assert_array_equal(idx[:, off:off + n].cpu().numpy().reshape((v.ndim,) + v.shape),
                                      oi[:, 0, 0])
        off += n


@pytest.mark.parametrize("nd,planes", [(2, False), (3, False), (3, True)])
@pytest.mark.parametrize("p", [0.9, 0.995])
def test_ragged_edt_vs_oracle(cuda, nd, planes, p):
    """planes: every axis of every 3-D item is at most 180 voxels, so the batch takes the
    fused plane passes (pass 0 per column, passes 1 + 2 per plane on chip); otherwise the
    per-line envelope passes (a 300-voxel axis)."""
    r = rng(10 * nd + int(p * 1000) + planes)
    if nd == 2:
        shapes = [(int(r.integers(1, 200)), int(r.integers(1, 300))) for _ in range(12)]
        shapes += [(1, 1), (1, 77), (300, 2), (40, 41), (33, 700)]  # 700: stack in the workspace
    elif planes:
        shapes = [(int(r.integers(1, 50)), int(r.integers(1, 70)), int(r.integers(1, 130))) for _ in range(10)]
        shapes += [(1, 1, 1), (1, 1, 180), (180, 2, 3), (3, 180, 5), (17, 33, 45), (20, 20, 20), (6, 7, 8)]
    else:
        shapes = [(int(r.integers(1, 30)), int(r.integers(1, 40)), int(r.integers(1, 60))) for _ in range(8)]
        shapes += [(1, 1, 1), (2, 3, 300), (20, 20, 20), (6, 7, 8)]
    items = [r.random(s) < p for s in shapes]
    items[-1][:] = True     # no background: the virtual site (-1, 0, ...)
    items[-2][:] = False    # all background
    rb = RaggedBatch.from_images([torch.from_numpy(v).cuda() for v in items])
    d, idx = ragged.euclidean_distance_transform(rb, return_indices=True)
    torch.cuda.synchronize()
    _check_edt(items, d, idx)
    # float32 input (nonzero = foreground), distances only
    d32 = ragged.euclidean_distance_transform(rb.map(lambda x: x.float()))
    assert torch.equal(d32.data, d.data)


def test_ragged_edt_graph_capture(cuda):
    r = rng(77)
    shapes = [(int(r.integers(8, 40)), int(r.integers(8, 40)), int(r.integers(8, 140))) for _ in range(6)]
    items = [r.random(s) < 0.9 for s in shapes]
    rb = RaggedBatch.from_images([torch.from_numpy(v).cuda() for v in items])
    eager = ragged.euclidean_distance_transform(rb, return_indices=True)
    graph, outs = ragged.capture(lambda b: ragged.euclidean_distance_transform(b, return_indices=True), rb)
    outs[0].data.zero_()
    outs[1].zero_()
    graph.replay()
    torch.cuda.synchronize()
    assert torch.equal(outs[0].data, eager[0].data) and torch.equal(outs[1], eager[1])
    _check_edt(items, outs[0], outs[1])
