"""Pin the grey-gradient oracle (numpy scatter) against float64 torch autograd (no GPU)."""

import numpy as np
import pytest
import torch

import oracle
from tests.helpers import rng, torch_grey_fp64


@pytest.mark.parametrize("mode", ["reflect", "constant", "nearest", "mirror", "wrap"])
@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("shape,ssize,origin", [((2, 1, 9, 11), (3, 3), (0, 0)),
                                                ((1, 2, 6, 5), (4, 3), (-1, 1)),
                                                ((1, 1, 3, 4, 5), (3, 2, 3), (0, 0, -1)),
                                                ((2, 1, 7), (5,), (2,))])
def test_oracle_gradient_matches_fp64_autograd(mode, dilation, shape, ssize, origin):
    r = rng(len(shape) * 10 + ssize[0])
    x = r.random(shape)
    st = r.random(ssize) * 0.1
    fp = r.random(ssize) < 0.7
    fp.flat[0] = True
    w = r.standard_normal(shape)
    out, arg = oracle.grey_arg(x, st, fp, origin, mode, 0.4, dilation)
    xt = torch.tensor(x, requires_grad=True)
    yt = torch_grey_fp64(xt, st, fp, origin, mode, 0.4, dilation)
    np.testing.assert_array_equal(yt.detach().numpy(), out)
    (yt * torch.from_numpy(w)).sum().backward()
    gin = oracle.grey_backward(w, arg, ssize, fp, origin, mode, dilation)
    np.testing.assert_allclose(gin, xt.grad.numpy(), rtol=1e-12, atol=1e-12)


def test_ties_go_to_the_first_tap():
    x = np.zeros((1, 1, 4, 4))
    out, arg = oracle.grey_arg(x, np.zeros((3, 3)), mode="nearest", dilation=True)
    assert (arg == 0).all()
