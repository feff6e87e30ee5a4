"""Binary morphology on bit-packed tiles (1-D / 2-D erosion, dilation with elements other
than full boxes; one-pass opening and closing; ragged batches): bit-exact against the
oracle's per-voxel tap loop, including items spanning several 32 x 128 tiles, offsets up
to the kernel's reach (16 rows, 32 columns), border_value and origins, and elements
beyond the reach (which compose the two operators)."""

import numpy as np
import pytest
import torch
from scipy import ndimage as ndi

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import RaggedBatch, _C, ragged
from tests.helpers import rng

pytestmark = pytest.mark.gpu

CROSS = ndi.generate_binary_structure(2, 1)


def _structures():
    r = rng(5)
    ring = np.ones((3, 3), bool)
    ring[1, 1] = False
    return {
        "cross": (CROSS, (0, 0)),
        "box3": (np.ones((3, 3), bool), (0, 0)),
        "ring": (ring, (0, 0)),
        "random5x7": (r.random((5, 7)) < 0.5, (1, -2)),
        "line65": (np.ones((1, 65), bool), (0, 0)),        # |dx| = 32: the reach
        "col33": (np.ones((33, 1), bool), (0, 0)),         # |dy| = 16: the reach
        "even4x6": (r.random((4, 6)) < 0.6, (0, 0)),
        "wide66": (np.ones((1, 66), bool), (0, 0)),        # beyond: the tap-loop path
    }


def _oracle(kind, x, st, origin, bv):
    ero = lambda v: oracle.binary(v, st, origin, bv, dilation=False)
    dil = lambda v: oracle.binary(v, st, origin, bv, dilation=True)
    return {"erosion": ero, "dilation": dil, "opening": lambda v: dil(ero(v)),
            "closing": lambda v: ero(dil(v))}[kind](x)


@pytest.mark.parametrize("kind", ["erosion", "dilation", "opening", "closing"])
@pytest.mark.parametrize("name", list(_structures()))
@pytest.mark.parametrize("bv", [False, True])
def test_uniform_2d_vs_oracle(cuda, kind, name, bv):
    st, origin = _structures()[name]
    x = rng(hash((kind, name, bv)) % 2**31).random((2, 2, 70, 300)) < 0.6
    fn = {"erosion": tm.binary_erosion, "dilation": tm.binary_dilation, "opening": tm.binary_opening,
          "closing": tm.binary_closing}[kind]
    got = fn(torch.from_numpy(x).cuda(), structure=torch.from_numpy(st), border_value=bv, origin=list(origin))
    np.testing.assert_array_equal(got.cpu().numpy(), _oracle(kind, x, st, origin, bv))


@pytest.mark.parametrize("shape", [(1, 1, 1, 1), (3, 1, 1, 200), (1, 2, 33, 129), (2, 1, 5, 1), (1, 1, 64, 128)])
@pytest.mark.parametrize("kind", ["opening", "closing"])
def test_uniform_shapes(cuda, shape, kind):
    x = rng(sum(shape)).random(shape) < 0.5
    st = np.ones((3, 5), bool)
    fn = tm.binary_opening if kind == "opening" else tm.binary_closing
    for bv in (False, True):
        got = fn(torch.from_numpy(x).cuda(), structure=torch.from_numpy(st), border_value=bv)
        np.testing.assert_array_equal(got.cpu().numpy(), _oracle(kind, x, st, (0, 0), bv))


def test_uniform_1d_and_float_input(cuda):
    r = rng(9)
    x = r.random((3, 2, 1000)) < 0.7
    st = np.array([1, 0, 1, 1, 1], bool)
    for kind, fn in (("erosion", tm.binary_erosion), ("opening", tm.binary_opening),
                     ("closing", tm.binary_closing)):
        got = fn(torch.from_numpy(x.astype(np.float32)).cuda(), structure=torch.from_numpy(st), origin=1)
        np.testing.assert_array_equal(got.cpu().numpy(), _oracle(kind, x, st, (1,), False))


def test_fused_kernel_is_used_and_matches_two_calls(cuda):
    """The one-pass call returns the reference's composition bit for bit; a structure
    beyond the reach makes the one-pass entry decline (None) instead of computing."""
    x = torch.from_numpy(rng(3).random((4, 1, 257, 513)) < 0.5).cuda()
    st = torch.from_numpy(CROSS)
    fused = _C.binary_composite("opening", x, st, [0, 0], False)
    assert fused is not None
    two = _C.binary_dilation_cuda(_C.binary_erosion_cuda(x, st, [0, 0], False), st, [0, 0], False)
    assert torch.equal(fused, two)
    assert _C.binary_composite("opening", x, torch.ones((1, 66), dtype=torch.bool), [0, 0], False) is None


@pytest.mark.parametrize("kind", ["erosion", "dilation", "opening", "closing"])
def test_ragged_vs_oracle(cuda, kind):
    r = rng(21 + len(kind))
    shapes = [(int(r.integers(1, 150)), int(r.integers(1, 400))) for _ in range(20)] + [(1, 1), (32, 128), (33, 129)]
    imgs = [r.random(s) < 0.55 for s in shapes]
    rb = RaggedBatch.from_images([torch.from_numpy(v).cuda() for v in imgs])
    for name in ("cross", "random5x7", "line65", "wide66"):
        st, origin = _structures()[name]
        fn = getattr(ragged, f"binary_{kind}")
        for bv in (False, True):
            out = fn(rb, torch.from_numpy(st), bv, list(origin))
            for v, g in zip(imgs, out.images()):
                exp = _oracle(kind, v[None, None], st, origin, bv)[0, 0]
                np.testing.assert_array_equal(g.cpu().numpy(), exp)


@pytest.mark.parametrize("kind", ["erosion", "dilation", "opening", "closing"])
@pytest.mark.parametrize("shape", [(2, 1, 9, 48), (1, 2, 200, 1040), (3, 1, 1, 4096), (1, 1, 130, 16)])
def test_uniform_row_walkers(cuda, kind, shape):
    """Rows of a multiple of 16 voxels take the row-streaming walkers (structures reaching
    at most 2 rows and 32 columns; others the tile kernel): 32-word strips, row blocks
    of 128, both border values, equal to the oracle."""
    x = rng(sum(shape) + len(kind)).random(shape) < 0.6
    fn = {"erosion": tm.binary_erosion, "dilation": tm.binary_dilation, "opening": tm.binary_opening,
          "closing": tm.binary_closing}[kind]
    nd = len(shape) - 2
    structs = [(CROSS, (0, 0)), (np.ones((5, 3), bool), (1, 0)), (np.ones((1, 65), bool), (0, 0)),
               (rng(4).random((5, 5)) < 0.5, (-1, 2))]
    if nd == 1:
        structs = [(np.array([1, 0, 1, 1, 1], bool), (1,)), (np.ones(65, bool), (0,))]
    for st, origin in structs:
        if not st.any():
            continue
        for bv in (False, True):
            got = fn(torch.from_numpy(x).cuda(), structure=torch.from_numpy(st), border_value=bv,
                     origin=list(origin))
            np.testing.assert_array_equal(got.cpu().numpy(), _oracle(kind, x, st, origin, bv))
