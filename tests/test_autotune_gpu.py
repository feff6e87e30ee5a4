"""Autotuner on the GPU: every variant of every tunable operator returns the built-in
choice's bits (tune() checks this before timing), the fastest is kept and cached."""

import numpy as np
import pytest
import torch

import oracle
import torchmorph_gb300 as tm
from torchmorph_gb300 import autotune

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _restore_table():
    yield
    for op in autotune.OPS:
        for cls in range(64):
            autotune.set_variant(op, cls, -1)


def _check(res, op, path):
    assert len(res["times_ms"]) == autotune.variants(op)
    assert all(t > 0 for t in res["times_ms"])
    assert autotune.get_variant(op, res["class"]) == res["best"]
    name = torch.cuda.get_device_name(torch.cuda.current_device())
    assert autotune.load_cache(path)["devices"][name][op][str(res["class"])] == res["best"]


def test_tune_grey_and_binary_boxes(cuda, tmp_path):
    path = str(tmp_path / "t.json")
    x = torch.rand((8, 1, 1024, 1024), device="cuda")
    res = autotune.tune_grey_dilation(x, size=3, path=path)
    _check(res, "grey_flat2d", path)
    # the binary boxes share the path: every variant agrees with the oracle
    xb = x > 0.5
    box = np.ones((3, 3), bool)
    exp = oracle.binary(xb[:1].cpu().numpy(), box, dilation=True)
    for v in range(autotune.variants("grey_flat2d")):
        autotune.set_variant("grey_flat2d", res["class"], v)  # xb has the same voxel count
        got = tm.binary_dilation(xb, structure=torch.from_numpy(box))
        np.testing.assert_array_equal(got[:1].cpu().numpy(), exp.astype(bool))


def test_tune_edt_and_chamfer(cuda, tmp_path):
    path = str(tmp_path / "t.json")
    x = torch.from_numpy(np.random.default_rng(0).random((2, 1, 64, 64, 128)) < 0.9).cuda()
    _check(autotune.tune_edt(x, path=path), "edt_3d", path)
    _check(autotune.tune_cdt(x, metric="taxicab", path=path), "cdt_3d", path)
    # the tuned choices still give the oracle's answer
    _, od, oi = oracle.edt(x.cpu().numpy())
    d, i = tm.euclidean_distance_transform(x, return_indices=True)
    np.testing.assert_array_equal(d.cpu().numpy(), od.astype(np.float32))
    np.testing.assert_array_equal(i.cpu().numpy(), oi)


def test_tune_sinkhorn(cuda, tmp_path):
    path = str(tmp_path / "t.json")
    r = np.random.default_rng(1)
    n, d = 40, 300
    pts = r.random((d, 2))
    cost = ((pts[:, None] - pts[None]) ** 2).sum(-1)
    a = torch.tensor(r.dirichlet(np.ones(d), n), dtype=torch.float32, device="cuda")
    b = torch.tensor(r.dirichlet(np.ones(d), n), dtype=torch.float32, device="cuda")
    C = torch.tensor(cost / cost.max(), dtype=torch.float32, device="cuda")
    for log_space in (False, True):
        _check(autotune.tune_sinkhorn(a, b, C, 0.1, max_iter=30, log_space=log_space, path=path),
               "sinkhorn_f32", path)
