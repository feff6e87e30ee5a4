"""Allocation-free EDT entry point (tm_edt_noalloc), called through the C ABI.

Some callers of this library cannot pass it device memory for scratch space
(their code path must not allocate, or they have no allocator to use), so
tm_edt_noalloc runs the EDT kernels on a fixed scratch area the library keeps
on the device.  This test checks that it returns exactly what the regular
entry point tm_edt returns, on two calls in a row that reuse the shared
scratch, and that a batch too large for the scratch area is refused.  It sits
in a file of its own, collected last.
"""

import ctypes

import numpy as np
import pytest
import torch

from torchmorph_gb300 import _lib

pytestmark = pytest.mark.gpu


def _edt_outputs(x):
    nd = x.dim() - 2
    d = torch.full(x.shape, -7.0, dtype=torch.float32, device=x.device)
    i = torch.full((nd, *x.shape), -7, dtype=torch.int32, device=x.device)
    s = torch.full(x.shape, -7, dtype=torch.int32, device=x.device)
    return d, i, s


def _regular(lib, x):
    d, i, s = _edt_outputs(x)
    batch, shape = x.shape[0] * x.shape[1], list(x.shape[2:])
    shp = _lib.i64_array(shape)
    nbytes = lib.tm_edt_workspace_size(batch, len(shape), shp, None)
    ws = torch.empty(max(1, nbytes), dtype=torch.uint8, device=x.device)
    st = lib.tm_edt(_lib.ptr(x), _lib.TM_U8, batch, len(shape), shp, None, _lib.ptr(d), _lib.ptr(i),
                    _lib.ptr(s), _lib.ptr(ws), nbytes, _lib.stream_of(x.device))
    _lib.check(st, "tm_edt")
    return d, i, s


def _noalloc(lib, x):
    d, i, s = _edt_outputs(x)
    batch, shape = x.shape[0] * x.shape[1], list(x.shape[2:])
    st = lib.tm_edt_noalloc(_lib.ptr(x), _lib.TM_U8, batch, len(shape), _lib.i64_array(shape),
                            _lib.ptr(d), _lib.ptr(i), _lib.ptr(s), _lib.stream_of(x.device))
    _lib.check(st, "tm_edt_noalloc")
    return d, i, s


@pytest.mark.parametrize("shape,p", [((2, 1, 96, 80, 64), 0.9), ((3, 2, 200, 256), 0.97)])
def test_noalloc_matches_regular_entry_point_twice(shape, p):
    if not torch.cuda.is_available():
        pytest.skip("CUDA device required")
    lib = _lib.load()
    rng = np.random.default_rng(123)
    # two different inputs back to back: the second call reuses the scratch
    # contents left by the first and must still be exact
    for seed in range(2):
        x = torch.from_numpy(rng.random(shape) < p).cuda()
        got = _noalloc(lib, x)
        exp = _regular(lib, x)
        torch.cuda.synchronize()
        for a, b in zip(got, exp):
            assert torch.equal(a, b)


def test_noalloc_shell_search_volume_vs_oracle():
    """A 128^3 Bernoulli(0.9) volume: rows of 128 voxels take the bitmap shell search
    (the benchmarked fast path) on the shared scratch.  Distances, indices and squared
    distances equal the oracle's on two calls in a row."""
    if not torch.cuda.is_available():
        pytest.skip("CUDA device required")
    import oracle

    lib = _lib.load()
    for seed in (0, 1):
        xn = np.random.default_rng(seed).random((1, 1, 128, 128, 128)) < 0.9
        d, i, s = _noalloc(lib, torch.from_numpy(xn).cuda())
        torch.cuda.synchronize()
        sq, od, oi = oracle.edt(xn)
        np.testing.assert_array_equal(d.cpu().numpy(), od.astype(np.float32))
        np.testing.assert_array_equal(i.cpu().numpy(), oi)
        np.testing.assert_array_equal(s.cpu().numpy(), sq.astype(np.int32))


def test_noalloc_rejects_batches_beyond_its_scratch():
    if not torch.cuda.is_available():
        pytest.skip("CUDA device required")
    lib = _lib.load()
    x = torch.zeros((6, 1, 128, 128, 128), dtype=torch.bool, device="cuda")  # ~12.6M voxels
    d = torch.empty(x.shape, dtype=torch.float32, device="cuda")
    st = lib.tm_edt_noalloc(_lib.ptr(x), _lib.TM_U8, 6, 3, _lib.i64_array([128, 128, 128]), _lib.ptr(d),
                            None, None, _lib.stream_of(x.device))
    assert st == 4  # TM_ERR_TOO_LARGE
    assert "scratch" in lib.tm_last_error().decode()
