"""Binary morphology parity: libtmcore vs the oracle and scipy.ndimage, bit-exact."""

import numpy as np
import pytest
import torch
from scipy import ndimage as ndi

import oracle
import torchmorph_gb300 as tm
from tests.helpers import per_item, rng

pytestmark = pytest.mark.gpu

# literal golden inputs of the reference's tests (test/test_binary.py:60-88)
CASE_2D = np.array([[[[0, 1, 0], [1, 1, 1], [0, 1, 0]]]], dtype=np.float32)
CASE_3D = np.zeros((2, 1, 5, 5, 5), dtype=bool)
CASE_3D[0, 0, 2:3, 2:4, 1:2] = True
CASE_4D = np.zeros((2, 1, 4, 4, 4, 4), dtype=bool)
CASE_4D[0, 0, 1:3, 1:2, 2:3] = True
HOLES_2D = np.zeros((1, 1, 5, 5), dtype=bool)
HOLES_2D[0, 0, 1:4, 1:4] = True
HOLES_2D[0, 0, 2, 2] = False
S2 = ndi.generate_binary_structure(2, 1)
S3_1 = ndi.generate_binary_structure(3, 2)
S3_2 = ndi.generate_binary_structure(3, 3)
S4 = ndi.generate_binary_structure(4, 4)
MASK_2D = np.array([[1, 1, 0], [1, 1, 1], [1, 1, 0]], dtype=bool)

OPS = [
    (tm.binary_erosion, ndi.binary_erosion),
    (tm.binary_dilation, ndi.binary_dilation),
    (tm.binary_opening, ndi.binary_opening),
    (tm.binary_closing, ndi.binary_closing),
]


def _t(x, dtype=None):
    return None if x is None else torch.as_tensor(x, dtype=dtype, device="cuda")


@pytest.mark.parametrize("ops", OPS, ids=["erosion", "dilation", "opening", "closing"])
@pytest.mark.parametrize(
    "x,st,it,origin,bv",
    [
        (CASE_2D, None, 1, 0, False),
        (CASE_2D, S2, 1, 0, False),
        (CASE_2D, None, 2, 0, False),
        (CASE_2D, None, -1, 0, False),
        (CASE_2D, None, 1, 1, True),
        (CASE_3D, None, 1, 0, False),
        (CASE_3D, S3_1, 1, 0, False),
        (CASE_3D, S3_2, 1, 1, True),
        (CASE_4D, S4, 1, 0, False),
        (CASE_4D, None, 2, 0, False),
    ],
)
def test_reference_cases_match_scipy(cuda, ops, x, st, it, origin, bv):
    ours, theirs = ops
    got = ours(_t(x, torch.float32), structure=_t(st, torch.bool), iterations=it, origin=origin,
               border_value=bv)
    exp = per_item(x, theirs, structure=st, iterations=it, origin=origin, border_value=bv)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("ops", OPS, ids=["erosion", "dilation", "opening", "closing"])
def test_mask(cuda, ops):
    ours, theirs = ops
    mask = torch.as_tensor(MASK_2D, device="cuda").expand(CASE_2D.shape)
    got = ours(_t(CASE_2D), mask=mask)
    exp = per_item(CASE_2D, theirs, mask=MASK_2D)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)


@pytest.mark.parametrize("dilation", [False, True])
@pytest.mark.parametrize("conn", [1, 2])
@pytest.mark.parametrize("bv", [False, True])
def test_random_2d_vs_oracle(cuda, dilation, conn, bv):
    r = rng(conn * 10 + bv)
    x = r.random((5, 2, 77, 131)) > 0.5
    st = ndi.generate_binary_structure(2, conn)
    op = tm.binary_dilation if dilation else tm.binary_erosion
    got = op(_t(x), structure=_t(st), border_value=bv)
    exp = oracle.binary(x, st, border_value=bv, dilation=dilation)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)


def test_config1_binary_vs_scipy(cuda):
    x = rng(0).random((8, 1, 256, 256)).astype(np.float32) > 0.5
    box = np.ones((3, 3), bool)
    got = tm.binary_dilation(_t(x), structure=_t(box))
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(x, ndi.binary_dilation, structure=box))
    got = tm.binary_dilation(_t(x))
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(x, ndi.binary_dilation))


def test_propagation_fill_holes_hit_or_miss(cuda):
    got = tm.binary_propagation(_t(CASE_2D), structure=_t(S2), origin=1, border_value=True)
    exp = per_item(CASE_2D, ndi.binary_propagation, structure=S2, origin=1, border_value=True)
    np.testing.assert_array_equal(got.cpu().numpy(), exp)
    got = tm.binary_fill_holes(_t(HOLES_2D))
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(HOLES_2D, ndi.binary_fill_holes))
    hit = ndi.generate_binary_structure(3, 1)[None, None]
    got = tm.binary_hit_or_miss(_t(hit))
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(hit, ndi.binary_hit_or_miss))


def test_until_stable_needs_many_iterations(cuda):
    """Iterate-until-stable runs its iterations in chunks with device-side change flags;
    a seed propagating through a 90 x 90 maze-like mask takes a few hundred iterations,
    i.e. several chunks.  Results equal scipy's fixed points."""
    r = rng(5)
    mask = r.random((2, 1, 90, 90)) < 0.75
    mask[:, :, ::6, :] = True  # corridors so that long paths exist
    seed = np.zeros_like(mask)
    seed[:, :, 0, 0] = True
    got = tm.binary_propagation(_t(seed), mask=_t(mask))
    exp = np.stack([ndi.binary_propagation(seed[b, 0], mask=mask[b, 0]) for b in range(2)])[:, None]
    np.testing.assert_array_equal(got.cpu().numpy(), exp)
    holes = r.random((2, 1, 90, 90)) < 0.55
    got = tm.binary_fill_holes(_t(holes))
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(holes, ndi.binary_fill_holes))
    got = tm.binary_erosion(_t(holes), iterations=-1)
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(holes, ndi.binary_erosion, iterations=-1))


@pytest.mark.parametrize("nd", [1, 8])
def test_dimension_range(cuda, nd):
    x = np.zeros((1, 1) + (2,) * nd, bool)
    x[(0, 0) + (0,) * nd] = True
    got = tm.binary_dilation(_t(x))
    np.testing.assert_array_equal(got.cpu().numpy(), per_item(x, ndi.binary_dilation))


def test_empty_structure_and_errors(cuda):
    x = _t(CASE_2D)
    z = torch.zeros((3, 3), dtype=torch.bool, device="cuda")
    assert tm.binary_erosion(x, structure=z).all()
    assert not tm.binary_dilation(x, structure=z).any()
    with pytest.raises(ValueError, match="origin dimension"):
        tm.binary_erosion(x, origin=(0, 0, 0))
    with pytest.raises(ValueError, match="invalid origin"):
        tm.binary_erosion(x, origin=2)
    with pytest.raises(ValueError, match="mask shape"):
        tm.binary_erosion(x, mask=torch.ones((3, 3), dtype=torch.bool, device="cuda"))
    with pytest.raises(ValueError, match="1 to 8"):
        tm.binary_dilation(torch.zeros((1, 1) + (1,) * 9, dtype=torch.bool, device="cuda"))
    assert not tm.binary_dilation(x.clone().requires_grad_()).requires_grad
