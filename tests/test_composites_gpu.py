"""One-pass grey opening, closing and top-hats (1-D / 2-D flat boxes) against the
composition of the two operators (the reference's definition) and the oracle: all
border modes, origins, even and odd windows, items smaller than the window and than a
tile, and tiles at item edges."""

import numpy as np
import pytest
import torch

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import _C
from tests.helpers import rng

pytestmark = pytest.mark.gpu

SHAPES = [(3, 1, 70, 300), (2, 2, 5, 7), (1, 1, 33, 129), (2, 1, 1, 40), (1, 1, 200, 3)]


def _composed(x, kind, size, mode, cval, origin):
    kw = dict(size=size, mode=mode, cval=cval, origin=origin)
    if kind in ("opening", "white_tophat"):
        op = tm.grey_dilation(tm.grey_erosion(x, **kw), **kw)
    else:
        op = tm.grey_erosion(tm.grey_dilation(x, **kw), **kw)
    if kind == "white_tophat":
        return x - op
    if kind == "black_tophat":
        return op - x
    return op


@pytest.mark.parametrize("kind", ["opening", "closing", "white_tophat", "black_tophat"])
@pytest.mark.parametrize("mode", ["reflect", "constant", "nearest", "mirror", "wrap"])
@pytest.mark.parametrize("size", [(3, 3), (4, 7), (15, 1), (1, 33)])
def test_one_pass_equals_composition(cuda, kind, mode, size):
    r = rng(hash((kind, mode, size)) % 1000)
    for shape in SHAPES:
        x = torch.from_numpy(r.random(shape).astype(np.float32)).cuda()
        origin = tuple(int(r.integers(-(k // 2), (k - 1) // 2 + 1)) for k in size)
        got = _C.grey_composite(kind, x, torch.zeros(size), torch.empty(0, dtype=torch.bool), list(origin),
                                {"constant": 0, "reflect": 1, "nearest": 2, "mirror": 3, "wrap": 4}[mode], 0.3)
        assert got is not None
        exp = _composed(x, kind, size, mode, 0.3, origin)
        torch.testing.assert_close(got, exp, rtol=0, atol=0)


def test_public_operators_take_the_one_pass_path_and_match_the_oracle(cuda):
    r = rng(2)
    x = r.random((2, 1, 90, 150)).astype(np.float32)
    t = torch.from_numpy(x).cuda()
    z = np.zeros((5, 5), np.float32)
    er = oracle.grey(x, z)
    op = oracle.grey(er, z, dilation=True)
    np.testing.assert_array_equal(tm.grey_opening(t, size=5).cpu().numpy(), op)
    np.testing.assert_array_equal(tm.white_tophat(t, size=5).cpu().numpy(), x - op)
    di = oracle.grey(x, z, dilation=True)
    cl = oracle.grey(di, z)
    np.testing.assert_array_equal(tm.grey_closing(t, size=5).cpu().numpy(), cl)
    np.testing.assert_array_equal(tm.black_tophat(t, size=5).cpu().numpy(), cl - x)
    # a flat structure with a value, 1-D items
    x1 = torch.from_numpy(r.random((3, 2, 500)).astype(np.float32)).cuda()
    st = torch.full((7,), 0.25)
    got = tm.grey_opening(x1, structure=st)
    exp = tm.grey_dilation(tm.grey_erosion(x1, structure=st), structure=st)
    assert torch.equal(got, exp)


def test_elements_outside_the_one_pass_kernel_compose(cuda):
    x = torch.rand((2, 1, 40, 50), device="cuda")
    fp = torch.tensor([[0, 1, 0], [1, 1, 1], [0, 1, 0]], dtype=torch.bool)
    assert _C.grey_composite("opening", x, torch.zeros(3, 3), fp, [0, 0], 1, 0.0) is None
    got = tm.grey_opening(x, footprint=fp)
    assert torch.equal(got, tm.grey_dilation(tm.grey_erosion(x, footprint=fp), footprint=fp))
    assert _C.grey_composite("closing", x, torch.zeros(35, 3), torch.empty(0, dtype=torch.bool), [0, 0], 1,
                             0.0) is None


@pytest.mark.parametrize("kind", ["opening", "closing", "white_tophat", "black_tophat"])
@pytest.mark.parametrize("size", [(3, 3), (5, 5)])
@pytest.mark.parametrize("mode", ["reflect", "constant", "wrap"])
def test_register_walkers_on_large_items(cuda, kind, size, mode):
    """3 x 3 and 5 x 5 windows: outputs whose footprint lies inside the item come from the
    register walkers (32-column strips, 64-row blocks, warp shuffles), the rest from the
    tile kernel; both with a structure value and every origin, equal to the composition."""
    r = rng(hash((kind, size, mode)) % 1000)
    x = torch.from_numpy(r.random((2, 1, 300, 700)).astype(np.float32)).cuda()
    codes = {"constant": 0, "reflect": 1, "nearest": 2, "mirror": 3, "wrap": 4}
    k = size[0]
    for oy in range(-(k // 2), (k - 1) // 2 + 1):
        for ox in (-(k // 2), 0, (k - 1) // 2):
            st = torch.full(size, 0.125)
            got = _C.grey_composite(kind, x, st, torch.empty(0, dtype=torch.bool), [oy, ox], codes[mode], 0.3)
            kw = dict(structure=st, mode=mode, cval=0.3, origin=(oy, ox))
            if kind in ("opening", "white_tophat"):
                op = tm.grey_dilation(tm.grey_erosion(x, **kw), **kw)
            else:
                op = tm.grey_erosion(tm.grey_dilation(x, **kw), **kw)
            exp = x - op if kind == "white_tophat" else (op - x if kind == "black_tophat" else op)
            assert torch.equal(got, exp), (oy, ox)
