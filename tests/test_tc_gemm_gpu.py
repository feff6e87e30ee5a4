"""tcgen05 error-compensated BF16 product (tm_gemm_bf16x3) vs float64 references."""

import numpy as np
import pytest
import torch

from torchmorph_gb300 import _lib

pytestmark = pytest.mark.gpu


def _gemm(a_hi, a_lo, b_hi, b_lo):
    lib = _lib.load()
    M, K = a_hi.shape
    N = b_hi.shape[0]
    d = torch.empty((M, N), dtype=torch.float32, device="cuda")
    _lib.check(lib.tm_gemm_bf16x3(_lib.ptr(a_hi), _lib.ptr(a_lo), _lib.ptr(b_hi), _lib.ptr(b_lo),
                                  _lib.ptr(d), M, N, K, _lib.stream_of(d.device)), "tm_gemm_bf16x3")
    torch.cuda.synchronize()
    assert lib.tm_device_error(1) == 0
    return d


def _split(x):
    hi = x.to(torch.bfloat16)
    lo = (x - hi.float()).to(torch.bfloat16)
    return hi.contiguous(), lo.contiguous()


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 256, 512), (384, 128, 1024),
                                   (128, 384, 192)])
def test_small_integers_are_exact(cuda, M, N, K):
    """Integer operands: every product and partial sum is exact in fp32, so D must be."""
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N * 3 + K)
    ints = lambda r, c: torch.randint(-4, 5, (r, c), generator=g).float()
    a_hi, a_lo, b_hi, b_lo = ints(M, K), ints(M, K), ints(N, K), ints(N, K)
    want = (a_hi.double() @ b_hi.double().T + a_lo.double() @ b_hi.double().T
            + a_hi.double() @ b_lo.double().T)
    bf = lambda t: t.to(torch.bfloat16).cuda().contiguous()
    got = _gemm(bf(a_hi), bf(a_lo), bf(b_hi), bf(b_lo))
    np.testing.assert_array_equal(got.cpu().double().numpy(), want.numpy())


def test_position_coded_operands(cuda):
    """One-hot rows pin the row/column mapping of the swizzled tiles and of TMEM."""
    M, N, K = 256, 256, 256
    a = torch.zeros(M, K)
    b = torch.zeros(N, K)
    a[torch.arange(M), torch.arange(M) % K] = 1.0
    b[torch.arange(N), (torch.arange(N) * 5) % K] = torch.arange(1, N + 1).float()
    zeros = lambda t: torch.zeros_like(t, dtype=torch.bfloat16, device="cuda")
    ah, bh = a.to(torch.bfloat16).cuda(), b.to(torch.bfloat16).cuda()
    got = _gemm(ah, zeros(a), bh, zeros(b))
    np.testing.assert_array_equal(got.cpu().numpy(), (a @ b.T).numpy())


@pytest.mark.parametrize("seed", [0, 1])
def test_fp32_accuracy_of_split_product(cuda, seed):
    """Positive fp32 operands (kernel-matrix-like): relative error ~1e-6, not bf16's 1e-3."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    M, N, K = 512, 256, 2048
    a = torch.exp(-8.0 * torch.rand(M, K, generator=g))
    b = torch.rand(N, K, generator=g)
    a_hi, a_lo = _split(a.cuda())
    b_hi, b_lo = _split(b.cuda())
    got = _gemm(a_hi, a_lo, b_hi, b_lo).double().cpu()
    want = a.double() @ b.double().T
    rel = ((got - want).abs() / want.abs()).max().item()
    assert rel < 2e-6, rel
    plain = (a_hi.double() @ b_hi.double().T).cpu()
    assert ((plain - want).abs() / want.abs()).max().item() > 10 * rel


def test_rejects_bad_shapes(cuda):
    lib = _lib.load()
    t = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
    d = torch.empty(128, 128, device="cuda")
    for M, N, K in [(100, 128, 64), (128, 96, 64), (128, 128, 48), (0, 128, 64)]:
        rc = lib.tm_gemm_bf16x3(_lib.ptr(t), _lib.ptr(t), _lib.ptr(t), _lib.ptr(t), _lib.ptr(d),
                                M, N, K, _lib.stream_of(d.device))
        assert rc == 1
