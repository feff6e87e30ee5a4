"""Ragged batches: one persistent launch per operator, bit-exact per image vs the oracle."""

import numpy as np
import pytest
import torch

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import RaggedBatch, ragged
from tests.helpers import rng

pytestmark = pytest.mark.gpu

CROSS = np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], bool)


def _shapes(seed, n=14, lo=1, hi=300):
    r = rng(seed)
    shapes = [(int(r.integers(lo, hi)), int(r.integers(lo, hi))) for _ in range(n)]
    return shapes + [(1, 1), (1, 37), (45, 1), (32, 128), (33, 129)]


def _batch(shapes, seed, binary=False):
    r = rng(seed)
    imgs = [r.random(s).astype(np.float32) for s in shapes]
    if binary:
        imgs = [im > 0.5 for im in imgs]
    return imgs, RaggedBatch.from_images([torch.from_numpy(im).cuda() for im in imgs])


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("mode", ["reflect", "constant", "nearest", "mirror", "wrap"])
@pytest.mark.parametrize("size", [(3, 3), (5, 5), (15, 15), (1, 3), (4, 9), (2, 1)])
def test_flat_grey_vs_oracle(cuda, dilation, mode, size):
    shapes = _shapes(hash((dilation, mode, size)) % 1000)
    imgs, rb = _batch(shapes, 1)
    r = rng(5)
    origin = (int(r.integers(-(size[0] // 2), (size[0] - 1) // 2 + 1)),
              int(r.integers(-(size[1] // 2), (size[1] - 1) // 2 + 1)))
    op = ragged.grey_dilation if dilation else ragged.grey_erosion
    out = op(rb, size=size, mode=mode, cval=0.3, origin=origin)
    torch.cuda.synchronize()
    assert out.shapes == rb.shapes
    for im, got in zip(imgs, out.images()):
        exp = oracle.grey(im[None, None], np.zeros(size, np.float32), origin=origin, mode=mode, cval=0.3,
                          dilation=dilation)[0, 0]
        np.testing.assert_array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("dilation", [False, True])
def test_nonflat_and_footprint_vs_oracle(cuda, dilation):
    shapes = _shapes(3, n=8)
    imgs, rb = _batch(shapes, 2)
    r = rng(4)
    st = r.random((3, 5)).astype(np.float32)
    fp = r.random((3, 5)) < 0.6
    fp[1, 2] = True
    op = ragged.grey_dilation if dilation else ragged.grey_erosion
    for mode in ["reflect", "constant", "wrap"]:
        out = op(rb, structure=torch.from_numpy(st), footprint=torch.from_numpy(fp), mode=mode, cval=-1.0)
        out2 = op(rb, footprint=torch.from_numpy(CROSS), mode=mode)
        for im, g1, g2 in zip(imgs, out.images(), out2.images()):
            e1 = oracle.grey(im[None, None], st, footprint=fp, mode=mode, cval=-1.0, dilation=dilation)[0, 0]
            e2 = oracle.grey(im[None, None], np.zeros((3, 3), np.float32), footprint=CROSS, mode=mode,
                             dilation=dilation)[0, 0]
            np.testing.assert_array_equal(g1.cpu().numpy(), e1)
            np.testing.assert_array_equal(g2.cpu().numpy(), e2)


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("border_value", [False, True])
@pytest.mark.parametrize("structure", ["cross", "box3", "box5x3"])
def test_binary_vs_oracle(cuda, dilation, border_value, structure):
    st = {"cross": CROSS, "box3": np.ones((3, 3), bool), "box5x3": np.ones((5, 3), bool)}[structure]
    imgs, rb = _batch(_shapes(11), 3, binary=True)
    op = ragged.binary_dilation if dilation else ragged.binary_erosion
    out = op(rb, structure=torch.from_numpy(st), border_value=border_value)
    for im, got in zip(imgs, out.images()):
        exp = oracle.binary(im[None, None], st, border_value=border_value, dilation=dilation)[0, 0]
        np.testing.assert_array_equal(got.cpu().numpy(), exp)


def test_matches_uniform_operators(cuda):
    """Composites per image equal the drop-in operators on image[None, None]."""
    imgs, rb = _batch(_shapes(21, n=6), 4)
    xb = rb.map(lambda x: x > 0.5)
    checks = [
        (ragged.grey_opening(rb, size=5), lambda t: tm.grey_opening(t, size=5)),
        (ragged.grey_closing(rb, size=(3, 7)), lambda t: tm.grey_closing(t, size=(3, 7))),
        (ragged.binary_opening(xb), lambda t: tm.binary_opening(t > 0.5)),
        (ragged.binary_closing(xb), lambda t: tm.binary_closing(t > 0.5)),
    ]
    for out, ref in checks:
        for im, got in zip(imgs, out.images()):
            exp = ref(torch.from_numpy(im).cuda()[None, None])[0, 0]
            assert torch.equal(got, exp)


def test_cuda_graph_replay_matches_eager(cuda):
    """The benchmark pipeline (erosion 5 and 15, binary opening of x > 0.5) captured once."""
    imgs, rb = _batch(_shapes(31, n=20, lo=32, hi=400), 5)

    def pipeline(b):
        return (ragged.grey_erosion(b, size=5), ragged.grey_erosion(b, size=15),
                ragged.binary_opening(b.map(lambda x: x > 0.5)))

    eager = pipeline(rb)
    graph, outs = ragged.capture(pipeline, rb)
    for o in outs:
        o.data.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for e, o in zip(eager, outs):
        assert torch.equal(e.data, o.data)
    # new input values, same buffers: replay recomputes
    rb.data.copy_(torch.rand_like(rb.data))
    graph.replay()
    for e, o in zip(pipeline(rb), outs):
        assert torch.equal(e.data, o.data)


def test_plan_shared_and_errors(cuda):
    imgs, rb = _batch([(10, 20), (7, 3)], 6)
    out = ragged.grey_erosion(rb, size=3)
    assert out.plan.data_ptr() == rb.plan.data_ptr()
    with pytest.raises(ValueError, match="float32"):
        ragged.grey_erosion(rb.map(lambda x: x > 0.5), size=3)
    with pytest.raises(ValueError, match="Unknown mode"):
        ragged.grey_erosion(rb, size=3, mode="bad")
    with pytest.raises(ValueError, match="invalid origin"):
        ragged.grey_erosion(rb, size=3, origin=2)
    with pytest.raises(RuntimeError, match="1..255"):
        ragged.grey_erosion(rb, size=(300, 3))
    with pytest.raises(ValueError, match="alias"):
        ragged.grey_erosion(rb, size=3, output=rb)
