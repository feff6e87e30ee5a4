"""Grey morphology parity: libtmcore vs the oracle and scipy.ndimage, bit-exact."""

import numpy as np
import pytest
import torch
from scipy import ndimage as ndi

import oracle
import torchmorph_gb300 as tm
from tests.helpers import per_item, rng

pytestmark = pytest.mark.gpu

# literal golden inputs of the reference's tests (test/test_grey.py:42-47)
CASE_2D = np.arange(1, 10, dtype=np.float32).reshape(1, 1, 3, 3)
CASE_3D = np.arange(2 * 1 * 4 * 4 * 4, dtype=np.float32).reshape(2, 1, 4, 4, 4)
CROSS = ndi.generate_binary_structure(2, 1)
ASYM = np.arange(9, dtype=np.float32).reshape(3, 3)

OPS = [
    (tm.grey_erosion, ndi.grey_erosion),
    (tm.grey_dilation, ndi.grey_dilation),
    (tm.grey_opening, ndi.grey_opening),
    (tm.grey_closing, ndi.grey_closing),
    (tm.morphological_gradient, ndi.morphological_gradient),
    (tm.morphological_laplace, ndi.morphological_laplace),
    (tm.white_tophat, ndi.white_tophat),
    (tm.black_tophat, ndi.black_tophat),
]
OP_IDS = ["erosion", "dilation", "opening", "closing", "gradient", "laplace", "white", "black"]


def _t(x, dtype=None):
    return None if x is None else torch.as_tensor(x, dtype=dtype, device="cuda")


@pytest.mark.parametrize("ops", OPS, ids=OP_IDS)
@pytest.mark.parametrize(
    "case",
    [
        (CASE_2D, 3, None, None, 0),
        (CASE_2D, (2, 3), None, None, 0),
        (CASE_2D, None, CROSS, None, 0),
        (CASE_2D, None, None, ASYM, 1),
        (CASE_2D, None, CROSS, CROSS.astype(np.float32), 0),
        (CASE_3D, 3, None, None, 0),
    ],
    ids=["size", "even_size", "footprint", "asym_structure_origin", "structure_footprint", "3d"],
)
def test_reference_cases_match_scipy(cuda, ops, case):
    ours, theirs = ops
    x, size, fp, st, origin = case
    got = ours(_t(x), size=size, footprint=_t(fp, torch.bool), structure=_t(st, torch.float32),
               origin=origin)
    exp = per_item(x, theirs, size=size, footprint=fp, structure=st, origin=origin)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("ops", OPS, ids=OP_IDS)
@pytest.mark.parametrize("mode,cval", [("reflect", 0.0), ("constant", 0.0), ("constant", 99.0),
                                       ("constant", -99.0), ("nearest", 0.0), ("mirror", 0.0),
                                       ("wrap", 0.0)])
def test_border_modes_match_scipy(cuda, ops, mode, cval):
    ours, theirs = ops
    got = ours(_t(CASE_2D), size=3, mode=mode, cval=cval)
    exp = per_item(CASE_2D, theirs, size=3, mode=mode, cval=cval)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("mode", ["reflect", "constant", "nearest", "mirror", "wrap"])
@pytest.mark.parametrize("size", [(1, 1), (3, 3), (1, 7), (5, 2), (15, 15), (9, 13), (16, 4)])
def test_flat_2d_random_vs_oracle(cuda, dilation, mode, size):
    r = rng(hash((dilation, mode, size)) % 2**32)
    x = r.random((3, 2, 67, 150)).astype(np.float32)
    origin = (r.integers(-(size[0] // 2), (size[0] - 1) // 2 + 1),
              r.integers(-(size[1] // 2), (size[1] - 1) // 2 + 1))
    op = tm.grey_dilation if dilation else tm.grey_erosion
    got = op(_t(x), size=size, mode=mode, cval=0.25, origin=origin)
    exp = oracle.grey(x, np.zeros(size, np.float32), origin=origin, mode=mode, cval=0.25,
                      dilation=dilation)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("shape,ssize", [((2, 1, 41), (5,)), ((1, 2, 9, 10, 11), (3, 3, 3)),
                                         ((1, 1, 5, 4, 6, 3), (3, 2, 3, 1)),
                                         ((2, 1, 30, 31), (4, 5))])
def test_nonflat_and_nd_vs_oracle(cuda, dilation, shape, ssize):
    r = rng(7)
    x = r.random(shape).astype(np.float32)
    st = r.random(ssize).astype(np.float32)
    fp = r.random(ssize) < 0.7
    fp.flat[0] = True
    op = tm.grey_dilation if dilation else tm.grey_erosion
    for mode in ["reflect", "constant", "mirror", "wrap", "nearest"]:
        got = op(_t(x), structure=_t(st), footprint=_t(fp, torch.bool), mode=mode, cval=-0.5)
        exp = oracle.grey(x, st, footprint=fp, mode=mode, cval=-0.5, dilation=dilation)
        np.testing.assert_array_equal(got.cpu().numpy(), exp)
        # flat N-D boxes go through the same operators
        got = op(_t(x), size=ssize, mode=mode)
        exp = oracle.grey(x, np.zeros(ssize, np.float32), mode=mode, dilation=dilation)
        np.testing.assert_array_equal(got.cpu().numpy(), exp)


def test_large_tap_table_is_chunked(cuda):
    r = rng(3)
    x = r.random((1, 1, 70, 80)).astype(np.float32)
    st = r.random((45, 61)).astype(np.float32)  # 2745 taps > one launch's table
    got = tm.grey_erosion(_t(x), structure=_t(st))
    exp = oracle.grey(x, st, dilation=False)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)


def test_config1_shape_vs_oracle(cuda):
    x = rng(0).random((8, 1, 256, 256)).astype(np.float32)
    got = tm.grey_dilation(_t(x), size=3)
    exp = oracle.grey(x, np.zeros((3, 3), np.float32), dilation=True)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(x, ndi.grey_dilation, size=3))


@pytest.mark.parametrize("op,value", [(tm.grey_erosion, np.inf), (tm.grey_dilation, -np.inf)])
def test_infinite_extrema(cuda, op, value):
    x = np.full((1, 1, 5, 5), value, np.float32)
    np.testing.assert_array_equal(op(_t(x), size=3).cpu().numpy(), x)


@pytest.mark.parametrize("ops", OPS, ids=OP_IDS)
def test_output_argument(cuda, ops):
    ours, theirs = ops
    x = _t(CASE_2D)
    out = torch.empty_like(x)
    res = ours(x, size=3, output=out)
    assert res is out
    np.testing.assert_array_equal(out.cpu().numpy(), per_item(CASE_2D, theirs, size=3))


def test_errors_and_contract(cuda):
    x = _t(CASE_2D)
    with pytest.raises(ValueError, match="output shape"):
        tm.grey_erosion(x, size=3, output=torch.empty((1, 1, 2, 2), device="cuda"))
    with pytest.raises(ValueError, match="same device"):
        tm.grey_erosion(x, size=3, output=torch.empty_like(x, device="cpu"))
    with pytest.raises(ValueError, match="spatial dimensions"):
        tm.grey_erosion(torch.ones((1, 1, *([2] * 9)), device="cuda"), size=3)
    with pytest.raises(ValueError, match="At least one"):
        tm.grey_erosion(x)
    with pytest.raises(ValueError, match="at least 3 dimensions"):
        tm.grey_erosion(torch.tensor([1.0, 2.0], device="cuda"), size=3)
    with pytest.raises(ValueError, match="Unknown mode"):
        tm.grey_erosion(x, size=3, mode="invalid")
    for o in (-2, 2):
        with pytest.raises(ValueError, match="invalid origin"):
            tm.grey_erosion(x, size=3, origin=o)
    for s in (0, -1, (3, 0)):
        with pytest.raises(ValueError, match="greater than zero"):
            tm.grey_erosion(x, size=s)
    xr = x.clone().requires_grad_()
    assert not tm.grey_dilation(xr, size=3).requires_grad


def test_current_stream_semantics(cuda):
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        torch.cuda._sleep(2_000_000)
        x = torch.arange(25, dtype=torch.float32, device="cuda").reshape(1, 1, 5, 5)
        res = tm.grey_dilation(x, size=3)
    stream.synchronize()
    np.testing.assert_array_equal(res.cpu().numpy(),
                                  per_item(x.cpu().numpy(), ndi.grey_dilation, size=3))


def test_deterministic(cuda):
    x = _t(rng(1).random((4, 1, 100, 90)).astype(np.float32))
    a = tm.grey_erosion(x, footprint=_t(CROSS, torch.bool))
    b = tm.grey_erosion(x, footprint=_t(CROSS, torch.bool))
    assert torch.equal(a, b)


def _device_error():
    from torchmorph_gb300 import _lib

    return _lib.load().tm_device_error(1)


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("mode", ["reflect", "constant", "wrap"])
@pytest.mark.parametrize("size", [(3, 3), (1, 5), (15, 15), (4, 9), (31, 2)])
def test_flat_2d_tma_tiles_vs_oracle(cuda, dilation, mode, size):
    """Images with 16-byte rows take the TMA path for every interior tile."""
    r = rng(hash((dilation, mode, size, 1)) % 2**32)
    x = r.random((3, 1, 150, 512)).astype(np.float32)
    origin = (r.integers(-(size[0] // 2), (size[0] - 1) // 2 + 1),
              r.integers(-(size[1] // 2), (size[1] - 1) // 2 + 1))
    op = tm.grey_dilation if dilation else tm.grey_erosion
    got = op(_t(x), size=size, mode=mode, cval=0.75, origin=origin)
    exp = oracle.grey(x, np.zeros(size, np.float32), origin=origin, mode=mode, cval=0.75,
                      dilation=dilation)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)
    assert _device_error() == 0


@pytest.mark.parametrize("dilation", [False, True])
def test_binary_box_tma_tiles_vs_oracle(cuda, dilation):
    x = rng(9).random((2, 2, 97, 384)) > 0.4
    st = np.ones((5, 3), bool)
    op = tm.binary_dilation if dilation else tm.binary_erosion
    got = op(_t(x), structure=_t(st))
    exp = oracle.binary(x, st, dilation=dilation)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)
    assert _device_error() == 0


ELEMENTS = {
    "box3": dict(size=3),
    "box3x5": dict(size=(3, 5)),
    "even4_origin": dict(size=(4, 4), origin=(-1, 1)),
    "nonflat": dict(structure=torch.tensor(rng(31).random((3, 3)) * 0.2, dtype=torch.float32)),
    "footprint": dict(footprint=torch.tensor((rng(32).random((5, 5)) < 0.6) | np.eye(5, dtype=bool))),
    "wide31": dict(size=(1, 31)),
    "too_many_taps": dict(size=(9, 9)),  # 81 taps: composed from the two operators
}


@pytest.mark.parametrize("kind", ["gradient", "laplace"])
@pytest.mark.parametrize("mode", ["reflect", "constant", "nearest", "mirror", "wrap"])
@pytest.mark.parametrize("elem", list(ELEMENTS))
def test_one_pass_composites_equal_two_operators(cuda, kind, mode, elem):
    """2-D gradient / laplace in one pass (elements of up to 64 taps spanning up to 31)
    equal the reference's formulas on the two operators bit for bit: d - e and
    (d + e) - 2 x in float32; flat gradients also equal scipy."""
    kw = dict(ELEMENTS[elem], mode=mode, cval=0.3)
    x = rng(hash((kind, mode, elem)) % 2**31).random((2, 2, 150, 300)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    got = getattr(tm, f"morphological_{kind}")(xt, **kw)
    d, e = tm.grey_dilation(xt, **kw), tm.grey_erosion(xt, **kw)
    exp = d - e if kind == "gradient" else d + e - 2 * xt
    assert torch.equal(got, exp)
    if kind == "gradient" and "size" in ELEMENTS[elem]:
        sk = {k: v for k, v in kw.items()}
        np.testing.assert_array_equal(got.cpu().numpy(), per_item(x, ndi.morphological_gradient, **sk))


def test_one_pass_composites_leave_3d_to_the_operators(cuda):
    x = torch.from_numpy(rng(33).random((1, 1, 20, 30, 40)).astype(np.float32)).cuda()
    for kind in ("gradient", "laplace"):
        got = getattr(tm, f"morphological_{kind}")(x, size=3)
        d, e = tm.grey_dilation(x, size=3), tm.grey_erosion(x, size=3)
        assert torch.equal(got, d - e if kind == "gradient" else d + e - 2 * x)
