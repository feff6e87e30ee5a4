"""Pin the CPU oracle against the committed golden fixtures (scipy.ndimage and the
reference's own float64 CPU Sinkhorn), so that the GPU parity tests inherit it."""

import os

import numpy as np
import pytest
from scipy import ndimage as ndi

import oracle

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


@pytest.mark.parametrize("name,dil", [("erosion", False), ("dilation", True)])
def test_grey_reference_cases(name, dil):
    c2, c3, asym = G["grey_case2"], G["grey_case3"], G["grey_asym"]
    z = lambda s: np.zeros(s, np.float32)  # noqa: E731
    cross = ndi.generate_binary_structure(2, 1)
    np.testing.assert_array_equal(oracle.grey(c2, z((3, 3)), dilation=dil), G[f"grey_{name}_case2_size3"])
    np.testing.assert_array_equal(oracle.grey(c2, z((2, 3)), dilation=dil), G[f"grey_{name}_case2_size23"])
    np.testing.assert_array_equal(oracle.grey(c2, z((3, 3)), footprint=cross, dilation=dil),
                                  G[f"grey_{name}_case2_cross"])
    np.testing.assert_array_equal(oracle.grey(c2, asym, origin=(1, 1), dilation=dil),
                                  G[f"grey_{name}_case2_asym_o1"])
    np.testing.assert_array_equal(oracle.grey(c3, z((3, 3, 3)), dilation=dil), G[f"grey_{name}_case3_size3"])
    for mode, cval in [("reflect", 0.0), ("constant", 0.0), ("constant", 99.0), ("constant", -99.0),
                       ("nearest", 0.0), ("mirror", 0.0), ("wrap", 0.0)]:
        np.testing.assert_array_equal(oracle.grey(c2, z((3, 3)), mode=mode, cval=cval, dilation=dil),
                                      G[f"grey_{name}_case2_{mode}_{int(cval)}"])


def test_grey_random():
    x, st, fp = G["grey_rand_x"], G["grey_rand_st"], G["grey_rand_fp"]
    np.testing.assert_array_equal(oracle.grey(x, st, footprint=fp), G["grey_rand_erosion"])
    np.testing.assert_array_equal(oracle.grey(x, st, footprint=fp, dilation=True), G["grey_rand_dilation"])
    np.testing.assert_array_equal(oracle.grey(x, np.zeros((5, 3), np.float32), mode="wrap", dilation=True),
                                  G["grey_rand_dilation_size5_wrap"])


def test_binary_cases():
    c2, c3 = G["bin_case2"], G["bin_case3"]
    cross2 = ndi.generate_binary_structure(2, 1)
    s31 = ndi.generate_binary_structure(3, 2)
    for name, dil in [("erosion", False), ("dilation", True)]:
        np.testing.assert_array_equal(oracle.binary(c2, cross2, dilation=dil), G[f"bin_{name}_case2"])
        np.testing.assert_array_equal(oracle.binary(c2, cross2, origin=(1, 1), border_value=True, dilation=dil),
                                      G[f"bin_{name}_case2_o1_bv1"])
        np.testing.assert_array_equal(oracle.binary(c3, s31, dilation=dil), G[f"bin_{name}_case3_s31"])
    x = G["bin_rand_x"]
    for conn in (1, 2):
        st = ndi.generate_binary_structure(2, conn)
        np.testing.assert_array_equal(oracle.binary(x, st), G[f"bin_rand_erosion_c{conn}"])
        np.testing.assert_array_equal(oracle.binary(x, st, border_value=True, dilation=True),
                                      G[f"bin_rand_dilation_c{conn}_bv1"])


@pytest.mark.parametrize("key", ["lattice1", "lattice2", "lattice3", "hd4", "hd5", "rand3", "allfg"])
def test_edt(key):
    x = G[f"dt_{key}"]
    sq, d, i = oracle.edt(x)
    np.testing.assert_array_equal(d, G[f"edt_{key}_d"])
    np.testing.assert_array_equal(i, G[f"edt_{key}_i"])
    np.testing.assert_array_equal(np.sqrt(sq.astype(np.float64)), G[f"edt_{key}_d"])


def test_edt_sampled():
    _, d, i = oracle.edt(G["dt_rand3"], sampling=(1.0, 1.0, 2.5))
    np.testing.assert_array_equal(d, G["edt_rand3_s_d"])
    np.testing.assert_array_equal(i, G["edt_rand3_s_i"])
    _, d, i = oracle.edt(G["dt_allfg"], sampling=(0.5, 1.5))
    np.testing.assert_array_equal(d, G["edt_allfg_s_d"])
    np.testing.assert_array_equal(i, G["edt_allfg_s_i"])


@pytest.mark.parametrize("metric", ["chessboard", "taxicab"])
@pytest.mark.parametrize("key", ["lattice1", "lattice2", "lattice3", "rand3"])
def test_cdt(metric, key):
    d, i = oracle.cdt(G[f"dt_{key}"], metric)
    np.testing.assert_array_equal(d, G[f"cdt_{metric}_{key}_d"])
    np.testing.assert_array_equal(i, G[f"cdt_{metric}_{key}_i"])


@pytest.mark.parametrize("metric", ["euclidean", "taxicab", "chessboard"])
@pytest.mark.parametrize("key", ["lattice1", "lattice2", "lattice3", "rand2"])
def test_bf(metric, key):
    d, i = oracle.bfdt(G[f"dt_{key}"], metric)
    np.testing.assert_array_equal(d, G[f"bf_{metric}_{key}_d"])
    np.testing.assert_array_equal(i, G[f"bf_{metric}_{key}_i"])


@pytest.mark.parametrize("log_space", [False, True])
@pytest.mark.parametrize("nd", ["1x4", "3x6", "2x16"])
def test_sinkhorn_vs_reference_cpu(log_space, nd):
    key = f"ot_{'log' if log_space else 'scal'}_{nd}"
    a, b, c = G[key + "_a"], G[key + "_b"], G[key + "_cost"]
    lu, lv, its = oracle.sinkhorn(a, b, c, 1.5, 300, log_space=log_space)
    assert its == 300
    np.testing.assert_allclose(lu, G[key + "_log_u"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(lv, G[key + "_log_v"], rtol=1e-10, atol=1e-10)
    dist, _, _ = oracle.sinkhorn_cost(c, lu, lv, 1.5)
    np.testing.assert_allclose(dist, G[key + "_dist"], rtol=1e-10, atol=1e-12)


def test_chamfer345_matches_closed_form():
    """Two-pass 3-4-5 chamfer equals min over backgrounds of |d|_1 + 2|d|_inf (brute force)."""
    r = np.random.default_rng(3)
    x = r.random((1, 1, 9, 10, 8)) < 0.93
    d, _ = oracle.cdt(x, "chamfer345")
    bg = np.argwhere(~x[0, 0])
    exp = np.empty(x.shape[2:], np.int64)
    for p in np.ndindex(*x.shape[2:]):
        diff = np.abs(bg - np.array(p))
        exp[p] = (diff.sum(1) + 2 * diff.max(1)).min()
    np.testing.assert_array_equal(d[0, 0], exp)


@pytest.mark.parametrize("nm", ["7x11", "20x13", "5x5"])
def test_pointcloud_sinkhorn_vs_reference_log_iterations(nm):
    key = f"pc_{nm}"
    x, y, eps, iters = G[key + "_x"], G[key + "_y"], float(G[key + "_eps"]), int(G[key + "_iters"])
    f, g, its, _ = oracle.pointcloud_sinkhorn(x, y, eps, iters)
    assert its == iters
    n, m = len(x), len(y)
    np.testing.assert_allclose(f / eps - np.log(n), G[key + "_log_u"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(g / eps - np.log(m), G[key + "_log_v"], rtol=1e-10, atol=1e-10)
