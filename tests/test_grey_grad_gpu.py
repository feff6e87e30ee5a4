"""Opt-in grey erosion/dilation backward: recorded taps vs the oracle, gradients vs the
float64 oracle / float64 torch autograd, and central finite differences (h = 1e-3)."""

import numpy as np
import pytest
import torch

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import _C
from tests.helpers import rng, torch_grey_fp64

pytestmark = pytest.mark.gpu

MODES = ["reflect", "constant", "nearest", "mirror", "wrap"]
CASES = [((2, 1, 37, 53), (3, 3), (0, 0)), ((1, 2, 20, 9), (4, 5), (-1, 2)),
         ((1, 1, 11, 12, 13), (3, 3, 3), (0, 0, 0)), ((2, 1, 40), (7,), (-3,)),
         ((1, 1, 3, 2), (5, 5), (0, 0)), ((1, 1, 64, 64), (15, 15), (0, 0)),
         # 2-D tiled kernels (128 x 32 tiles): interior and border tiles, a shifted
         # origin, the widest tap extent they take (31) and a 2-D case they do not (33)
         ((1, 2, 150, 420), (3, 3), (0, 0)), ((2, 1, 131, 300), (9, 7), (2, -1)),
         ((1, 1, 100, 330), (1, 31), (0, 3)), ((1, 1, 70, 290), (33, 1), (0, 0))]


def _element(ssize, seed, flat):
    r = rng(seed)
    st = np.zeros(ssize, np.float32) if flat else (r.random(ssize) * 0.1).astype(np.float32)
    fp = np.ones(ssize, bool) if flat else r.random(ssize) < 0.7
    fp.flat[0] = True
    return st, fp


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("flat", [True, False])
@pytest.mark.parametrize("case", CASES, ids=[str(c[1]) for c in CASES])
def test_arg_forward_and_backward_vs_oracle(cuda, mode, dilation, flat, case):
    shape, ssize, origin = case
    r = rng(hash((mode, dilation, flat, ssize)) % 2**31)
    x = r.random(shape).astype(np.float32)
    st, fp = _element(ssize, 3, flat)
    stt, fpt = torch.from_numpy(st), torch.from_numpy(fp) if not flat else torch.empty(0, dtype=torch.bool)
    fn = _C.grey_dilation_arg if dilation else _C.grey_erosion_arg
    out, arg = fn(torch.from_numpy(x).cuda(), stt, fpt, list(origin), oracle._MODES[mode], 0.4)
    exp_out, exp_arg = oracle.grey_arg(x, st, None if flat else fp, origin, mode, 0.4, dilation)
    np.testing.assert_array_equal(out.cpu().numpy(), exp_out)
    np.testing.assert_array_equal(arg.cpu().numpy(), exp_arg)
    # the value equals the plain forward operator's, bit for bit
    plain = (_C.grey_dilation_cuda if dilation else _C.grey_erosion_cuda)(
        torch.from_numpy(x).cuda(), stt, fpt, list(origin), oracle._MODES[mode], 0.4)
    assert torch.equal(out, plain)
    g = r.standard_normal(shape).astype(np.float32)
    gin = _C.grey_morphology_backward(torch.from_numpy(g).cuda(), arg, list(ssize), fpt, list(origin),
                                      oracle._MODES[mode], dilation)
    exp = oracle.grey_backward(g, exp_arg, ssize, None if flat else fp, origin, mode, dilation)
    # fp32 sums of up to (taps) gradients against the float64 scatter
    np.testing.assert_allclose(gin.cpu().numpy(), exp, rtol=2e-5, atol=1e-5)


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("mode", ["reflect", "constant", "mirror"])
def test_autograd_vs_fp64_torch(cuda, dilation, mode):
    r = rng(17)
    x = r.random((2, 3, 31, 29))
    w = r.standard_normal(x.shape)
    xg = torch.tensor(x, dtype=torch.float32, device="cuda", requires_grad=True)
    op = tm.grey_dilation if dilation else tm.grey_erosion
    y = op(xg, size=(3, 5), mode=mode, cval=0.5, differentiable=True)
    assert y.requires_grad
    (y * torch.tensor(w, dtype=torch.float32, device="cuda")).sum().backward()
    x64 = torch.tensor(x.astype(np.float32).astype(np.float64), requires_grad=True)
    y64 = torch_grey_fp64(x64, np.zeros((3, 5)), None, None, mode, 0.5, dilation)
    (y64 * torch.from_numpy(w)).sum().backward()
    np.testing.assert_allclose(y.detach().cpu().numpy(), y64.detach().numpy(), rtol=0, atol=1e-7)
    np.testing.assert_allclose(xg.grad.cpu().numpy(), x64.grad.numpy(), rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("op_name", ["grey_dilation", "grey_erosion", "grey_opening",
                                     "morphological_gradient"])
def test_central_finite_differences(cuda, op_name):
    """Inputs are a permutation of a grid spaced 1e-2, so no tap order changes within
    h = 1e-3 and the central difference of the float64 forward is exact."""
    r = rng(23)
    shape = (1, 1, 12, 14)
    x = (r.permutation(np.prod(shape)).reshape(shape) * 1e-2).astype(np.float32)
    w = r.standard_normal(shape)
    xg = torch.tensor(x, device="cuda", requires_grad=True)
    y = getattr(tm, op_name)(xg, size=3, differentiable=True)
    (y * torch.tensor(w, dtype=torch.float32, device="cuda")).sum().backward()

    def f64(v):
        vt = torch.tensor(v, dtype=torch.float64)
        ero = lambda t: torch_grey_fp64(t, np.zeros((3, 3)), dilation=False)
        dil = lambda t: torch_grey_fp64(t, np.zeros((3, 3)), dilation=True)
        res = {"grey_dilation": dil, "grey_erosion": ero, "grey_opening": lambda t: dil(ero(t)),
               "morphological_gradient": lambda t: dil(t) - ero(t)}[op_name](vt)
        return float((res.numpy() * w).sum())

    h = 1e-3
    fd = np.zeros(shape)
    xd = x.astype(np.float64)
    for idx in np.ndindex(*shape):
        xp, xm = xd.copy(), xd.copy()
        xp[idx] += h
        xm[idx] -= h
        fd[idx] = (f64(xp) - f64(xm)) / (2 * h)
    np.testing.assert_allclose(xg.grad.cpu().numpy(), fd, rtol=1e-4, atol=1e-4)


def test_ties_route_to_the_first_tap(cuda):
    x = torch.zeros((1, 1, 6, 6), device="cuda", requires_grad=True)
    y = tm.grey_dilation(x, size=3, mode="nearest", differentiable=True)
    y.sum().backward()
    out, arg = oracle.grey_arg(np.zeros((1, 1, 6, 6), np.float32), np.zeros((3, 3), np.float32),
                               mode="nearest", dilation=True)
    exp = oracle.grey_backward(np.ones((1, 1, 6, 6)), arg, (3, 3), mode="nearest", dilation=True)
    np.testing.assert_array_equal(x.grad.cpu().numpy(), exp)


def test_default_is_not_differentiable_and_limits(cuda):
    x = torch.rand((1, 1, 8, 8), device="cuda", requires_grad=True)
    assert not tm.grey_dilation(x, size=3).requires_grad
    with torch.no_grad():
        assert not tm.grey_dilation(x, size=3, differentiable=True).requires_grad
    with pytest.raises(RuntimeError, match="255"):
        tm.grey_dilation(x, size=16, differentiable=True)
    x4 = torch.rand((1, 1, 3, 3, 3, 3), device="cuda", requires_grad=True)
    with pytest.raises(RuntimeError, match="1-3 spatial"):
        tm.grey_dilation(x4, size=2, differentiable=True)
