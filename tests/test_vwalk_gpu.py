"""Float4 register walkers (centred 3 x 3 and 5 x 5 flat windows on float32 items whose
rows are a multiple of 4 voxels): grey erosion / dilation, gradient, laplace and the
one-pass opening, closing and top-hats against the oracle, with the edge lanes' border
mapping and the frame kernel for the outputs the walkers leave.  Widths around the
120-column strip step, heights from one row (mapped rows) to the two-stage limit, every
border mode (wrap leaves the side columns to the frame kernel), a structure value,
infinities."""

import numpy as np
import pytest
import torch

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import _C
from tests.helpers import rng

pytestmark = pytest.mark.gpu

MODES = {"constant": 0, "reflect": 1, "nearest": 2, "mirror": 3, "wrap": 4}
# W = 16 (one strip), 124 / 128 / 132 (one or two strips), 252 / 256, 1000; H at 2 * lag + 1
SHAPES = [(2, 1, 5, 16), (1, 1, 9, 20), (1, 2, 40, 124), (2, 1, 11, 128), (1, 1, 64, 132), (3, 1, 17, 252),
          (1, 1, 130, 256), (1, 1, 37, 1000), (1, 1, 4, 64), (1, 1, 70, 18), (1, 1, 1, 16), (2, 1, 2, 32),
          (1, 1, 3, 248)]


def _values(r, shape):
    x = r.random(shape).astype(np.float32)
    x.flat[:: 97] = np.inf
    x.flat[5:: 89] = -np.inf
    return x


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("k", [3, 5])
@pytest.mark.parametrize("mode", list(MODES))
def test_single_operator_vs_oracle(cuda, dilation, k, mode):
    r = rng(k * 10 + int(dilation) + len(mode))
    for shape in SHAPES:
        x = _values(r, shape)
        for sval in (0.0, 0.25):
            st = np.full((k, k), sval, np.float32)
            fn = tm.grey_dilation if dilation else tm.grey_erosion
            got = fn(torch.from_numpy(x).cuda(), structure=torch.from_numpy(st), mode=mode, cval=0.7)
            exp = oracle.grey(x, st, mode=mode, cval=0.7, dilation=dilation)
            np.testing.assert_array_equal(got.cpu().numpy(), exp, err_msg=str((shape, sval)))


@pytest.mark.parametrize("kind", ["opening", "closing", "white_tophat", "black_tophat"])
@pytest.mark.parametrize("k", [3, 5])
@pytest.mark.parametrize("mode", list(MODES))
def test_one_pass_vs_oracle(cuda, kind, k, mode):
    r = rng(k * 100 + len(kind) + len(mode))
    for shape in SHAPES:
        x = _values(r, shape) if mode != "wrap" else r.random(shape).astype(np.float32)
        st = np.full((k, k), 0.125, np.float32)
        got = _C.grey_composite(kind, torch.from_numpy(x).cuda(), torch.from_numpy(st),
                                torch.empty(0, dtype=torch.bool), [0, 0], MODES[mode], 0.3)
        assert got is not None
        first_max = kind in ("closing", "black_tophat")
        a = oracle.grey(x, st, mode=mode, cval=0.3, dilation=first_max)
        op = oracle.grey(a, st, mode=mode, cval=0.3, dilation=not first_max)
        exp = x - op if kind == "white_tophat" else (op - x if kind == "black_tophat" else op)
        np.testing.assert_array_equal(got.cpu().numpy(), exp, err_msg=str(shape))


def test_walker_declines_unaligned_and_offset_items(cuda):
    """Rows that are not a multiple of 4 voxels, a storage offset that breaks 16-byte
    alignment, and off-centre origins take the tile kernels: same results."""
    r = rng(3)
    x = r.random((1, 1, 50, 203)).astype(np.float32)
    st = np.zeros((3, 3), np.float32)
    got = tm.grey_erosion(torch.from_numpy(x).cuda(), size=3)
    np.testing.assert_array_equal(got.cpu().numpy(), oracle.grey(x, st))
    big = torch.from_numpy(r.random(1 + 50 * 200).astype(np.float32)).cuda()
    view = big[1:].view(1, 1, 50, 200)
    got = tm.grey_dilation(view, size=3)
    np.testing.assert_array_equal(got.cpu().numpy(), oracle.grey(view.cpu().numpy(), st, dilation=True))
    x = r.random((1, 1, 60, 256)).astype(np.float32)
    got = tm.grey_erosion(torch.from_numpy(x).cuda(), size=3, origin=(1, -1))
    np.testing.assert_array_equal(got.cpu().numpy(), oracle.grey(x, st, origin=(1, -1)))


@pytest.mark.parametrize("kind", ["gradient", "laplace"])
@pytest.mark.parametrize("k", [3, 5])
@pytest.mark.parametrize("mode", list(MODES))
def test_gradient_and_laplace_vs_oracle(cuda, kind, k, mode):
    """Both extrema in one walk: dilation - erosion and (dilation + erosion) - 2 x,
    rounded like the reference's elementwise ops on the two operator images."""
    r = rng(k + len(kind) + len(mode))
    fn = tm.morphological_gradient if kind == "gradient" else tm.morphological_laplace
    for shape in SHAPES:
        x = r.random(shape).astype(np.float32) * 8 - 4
        for sval in (0.0, 0.375):
            st = np.full((k, k), sval, np.float32)
            got = fn(torch.from_numpy(x).cuda(), structure=torch.from_numpy(st), mode=mode, cval=0.5)
            d = oracle.grey(x, st, mode=mode, cval=0.5, dilation=True)
            e = oracle.grey(x, st, mode=mode, cval=0.5)
            exp = d - e if kind == "gradient" else (d + e) - np.float32(2) * x
            np.testing.assert_array_equal(got.cpu().numpy(), exp, err_msg=str((shape, sval)))


def _gather_f32(g, arg, k, dilation):
    """float32 gather in tap order for pixels no border mapping reaches (rows and
    columns in [h + 1, n - 1 - h)): the walker's sums, bit for bit."""
    h = k // 2
    B, C, H, W = g.shape
    acc = np.zeros_like(g)
    for t in range(k * k):
        i, j = divmod(t, k)
        dy, dx = (h - i, h - j) if dilation else (i - h, j - h)
        # output o = p - (dy, dx)
        gs = np.zeros_like(g)
        as_ = np.full(arg.shape, 255, np.uint8)
        ys, ye = max(0, dy), H + min(0, dy)
        xs, xe = max(0, dx), W + min(0, dx)
        gs[..., ys:ye, xs:xe] = g[..., ys - dy:ye - dy, xs - dx:xe - dx]
        as_[..., ys:ye, xs:xe] = arg[..., ys - dy:ye - dy, xs - dx:xe - dx]
        acc = np.where(as_ == t, acc + gs, acc).astype(np.float32)
    return acc[..., h + 1:H - 1 - h, h + 1:W - 1 - h]


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("k", [3, 5])
@pytest.mark.parametrize("mode", list(MODES))
def test_arg_forward_and_backward_walkers(cuda, dilation, k, mode):
    """Forward with argument (first tap attaining the extremum, raster order) and the
    gather backward: values and arguments bit-exact vs the oracle, gradients vs the
    float64 oracle and, away from the border, bit-exact vs a float32 gather in tap order.
    Quantised values make ties common."""
    r = rng(k * 7 + int(dilation) + len(mode))
    for shape in SHAPES:
        x = (np.floor(r.random(shape) * 6) / 4).astype(np.float32)
        st = np.full((k, k), 0.125, np.float32)
        fn = _C.grey_dilation_arg if dilation else _C.grey_erosion_arg
        out, arg = fn(torch.from_numpy(x).cuda(), torch.from_numpy(st), torch.empty(0, dtype=torch.bool), [0, 0],
                      MODES[mode], 0.3)
        exp_out, exp_arg = oracle.grey_arg(x, st, None, (0, 0), mode, 0.3, dilation)
        np.testing.assert_array_equal(out.cpu().numpy(), exp_out, err_msg=str(shape))
        np.testing.assert_array_equal(arg.cpu().numpy(), exp_arg, err_msg=str(shape))
        g = r.standard_normal(shape).astype(np.float32)
        gin = _C.grey_morphology_backward(torch.from_numpy(g).cuda(), arg, [k, k],
                                          torch.empty(0, dtype=torch.bool), [0, 0], MODES[mode], dilation)
        gin = gin.cpu().numpy()
        exp = oracle.grey_backward(g, exp_arg, (k, k), None, (0, 0), mode, dilation)
        np.testing.assert_allclose(gin, exp, rtol=2e-5, atol=1e-5, err_msg=str(shape))
        h = k // 2
        np.testing.assert_array_equal(gin[..., h + 1:shape[2] - 1 - h, h + 1:shape[3] - 1 - h],
                                      _gather_f32(g, exp_arg, k, dilation), err_msg=str(shape))
