"""Regenerate the golden fixtures under tests/golden/ (run in a container that has
scipy and the reference checkout; the fixtures themselves are committed).

Sources
  * scipy.ndimage (the oracle the reference's own tests use) on the literal
    inputs of the reference's tests -- test/test_grey.py:42-47,
    test/test_binary.py:60-88, test/test_distance_transform.py:13-24,302-320 --
    and on seeded random volumes that pin the tie rules;
  * the reference's own CPU Sinkhorn (torchmorph/optimal_transport.py,
    imported from the reference checkout) in float64 on the inputs of
    test/test_optimal_transport.py:34-36.

Usage:  python tests/golden/make_golden.py [/path/to/reference]
"""

from __future__ import annotations

import importlib.util
import os
import sys

import numpy as np
from scipy import ndimage as ndi

HERE = os.path.dirname(os.path.abspath(__file__))


def per_item(x, fn, **kw):
    s = x.shape[2:]
    out = [np.asarray(fn(t, **kw)) for t in x.reshape(-1, *s)]
    return np.stack(out).reshape(x.shape[:2] + out[0].shape)


def per_item_idx(x, fn, **kw):
    s = x.shape[2:]
    res = [fn(t, return_indices=True, **kw) for t in x.reshape(-1, *s)]
    d = np.stack([r[0] for r in res]).reshape(x.shape)
    i = np.stack([r[1] for r in res], axis=1).reshape((len(s),) + x.shape)
    return d, i


def grey_cases(out):
    case2 = np.arange(1, 10, dtype=np.float32).reshape(1, 1, 3, 3)
    case3 = np.arange(2 * 1 * 4 * 4 * 4, dtype=np.float32).reshape(2, 1, 4, 4, 4)
    cross = ndi.generate_binary_structure(2, 1)
    asym = np.arange(9, dtype=np.float32).reshape(3, 3)
    out["grey_case2"] = case2
    out["grey_case3"] = case3
    out["grey_asym"] = asym
    for name, fn in [("erosion", ndi.grey_erosion), ("dilation", ndi.grey_dilation)]:
        out[f"grey_{name}_case2_size3"] = per_item(case2, fn, size=3)
        out[f"grey_{name}_case2_size23"] = per_item(case2, fn, size=(2, 3))
        out[f"grey_{name}_case2_cross"] = per_item(case2, fn, footprint=cross)
        out[f"grey_{name}_case2_asym_o1"] = per_item(case2, fn, structure=asym, origin=1)
        out[f"grey_{name}_case3_size3"] = per_item(case3, fn, size=3)
        for mode, cval in [("reflect", 0.0), ("constant", 0.0), ("constant", 99.0),
                           ("constant", -99.0), ("nearest", 0.0), ("mirror", 0.0), ("wrap", 0.0)]:
            out[f"grey_{name}_case2_{mode}_{int(cval)}"] = per_item(case2, fn, size=3, mode=mode,
                                                                    cval=cval)
    r = np.random.default_rng(11)
    x = r.random((2, 1, 23, 29)).astype(np.float32)
    st = r.random((3, 4)).astype(np.float32)
    fp = r.random((3, 4)) < 0.6
    out["grey_rand_x"] = x
    out["grey_rand_st"] = st
    out["grey_rand_fp"] = fp
    out["grey_rand_erosion"] = per_item(x, ndi.grey_erosion, structure=st, footprint=fp)
    out["grey_rand_dilation"] = per_item(x, ndi.grey_dilation, structure=st, footprint=fp)
    out["grey_rand_dilation_size5_wrap"] = per_item(x, ndi.grey_dilation, size=(5, 3), mode="wrap")


def binary_cases(out):
    case2 = np.array([[[[0, 1, 0], [1, 1, 1], [0, 1, 0]]]], dtype=bool)
    case3 = np.zeros((2, 1, 5, 5, 5), dtype=bool)
    case3[0, 0, 2:3, 2:4, 1:2] = True
    s31 = ndi.generate_binary_structure(3, 2)
    out["bin_case2"] = case2
    out["bin_case3"] = case3
    for name, fn in [("erosion", ndi.binary_erosion), ("dilation", ndi.binary_dilation)]:
        out[f"bin_{name}_case2"] = per_item(case2, fn)
        out[f"bin_{name}_case2_o1_bv1"] = per_item(case2, fn, origin=1, border_value=True)
        out[f"bin_{name}_case3_s31"] = per_item(case3, fn, structure=s31)
    r = np.random.default_rng(12)
    x = r.random((2, 1, 19, 23)) < 0.5
    out["bin_rand_x"] = x
    for conn in (1, 2):
        st = ndi.generate_binary_structure(2, conn)
        out[f"bin_rand_erosion_c{conn}"] = per_item(x, ndi.binary_erosion, structure=st)
        out[f"bin_rand_dilation_c{conn}_bv1"] = per_item(x, ndi.binary_dilation, structure=st,
                                                         border_value=True)


def distance_cases(out):
    def lattice(shape):
        v = np.ones(shape, np.float32)
        v[(slice(None), slice(None), *[slice(None, None, 2)] * (len(shape) - 2))] = 0
        return v

    for nd, shape in [(1, (2, 1, 7)), (2, (2, 1, 5, 6)), (3, (1, 2, 4, 5, 6))]:
        x = lattice(shape)
        out[f"dt_lattice{nd}"] = x
        out[f"edt_lattice{nd}_d"], out[f"edt_lattice{nd}_i"] = per_item_idx(x, ndi.distance_transform_edt)
        for m in ("chessboard", "taxicab"):
            out[f"cdt_{m}_lattice{nd}_d"], out[f"cdt_{m}_lattice{nd}_i"] = per_item_idx(
                x, ndi.distance_transform_cdt, metric=m)
        for m in ("euclidean", "taxicab", "chessboard"):
            out[f"bf_{m}_lattice{nd}_d"], out[f"bf_{m}_lattice{nd}_i"] = per_item_idx(
                x, ndi.distance_transform_bf, metric=m)
    # high-dimensional random inputs of test_distance_transform.py:302-320
    rng42 = np.random.default_rng(42)
    for nd in (4, 5):
        x = rng42.integers(0, 2, size=(2, 2, *([2] * nd))).astype(np.float32)
        out[f"dt_hd{nd}"] = x
        out[f"edt_hd{nd}_d"], out[f"edt_hd{nd}_i"] = per_item_idx(x, ndi.distance_transform_edt)
    # tie-rule pins: random volumes with many equidistant backgrounds
    r = np.random.default_rng(13)
    x = r.random((2, 1, 15, 17, 11)) < 0.9
    out["dt_rand3"] = x
    out["edt_rand3_d"], out["edt_rand3_i"] = per_item_idx(x, ndi.distance_transform_edt)
    out["edt_rand3_s_d"], out["edt_rand3_s_i"] = per_item_idx(x, ndi.distance_transform_edt,
                                                              sampling=(1.0, 1.0, 2.5))
    for m in ("chessboard", "taxicab"):
        out[f"cdt_{m}_rand3_d"], out[f"cdt_{m}_rand3_i"] = per_item_idx(
            x, ndi.distance_transform_cdt, metric=m)
    y = r.random((2, 1, 13, 14)) < 0.85
    out["dt_rand2"] = y
    for m in ("euclidean", "taxicab", "chessboard"):
        out[f"bf_{m}_rand2_d"], out[f"bf_{m}_rand2_i"] = per_item_idx(y, ndi.distance_transform_bf,
                                                                      metric=m)
    z = np.ones((1, 1, 3, 4), np.float32)
    out["dt_allfg"] = z
    out["edt_allfg_d"], out["edt_allfg_i"] = per_item_idx(z, ndi.distance_transform_edt)
    out["edt_allfg_s_d"], out["edt_allfg_s_i"] = per_item_idx(z, ndi.distance_transform_edt,
                                                              sampling=(0.5, 1.5))


def sinkhorn_cases(out, ref_root):
    path = os.path.join(ref_root, "torchmorph", "optimal_transport.py")
    spec = importlib.util.spec_from_file_location("ref_optimal_transport", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)  # imports torch only; the CPU path needs no extension
    import torch

    def make_positive(shape, seed):
        g = torch.Generator(device="cpu").manual_seed(seed)
        return torch.rand(shape, generator=g, device="cpu") + 0.1

    for log_space in (False, True):
        for n, d in [(1, 4), (3, 6), (2, 16)]:
            solver = mod.SinkhornSolver(epsilon=1.5, max_iter=300, log_space=log_space)
            src = make_positive((n, d), 11).double()
            tgt = make_positive((n, d), 23).double()
            a, b, cost = solver.data_preprocess(src, tgt)
            log_u, log_v = solver._iterate(a, b, cost)
            key = f"ot_{'log' if log_space else 'scal'}_{n}x{d}"
            out[key + "_a"] = a.numpy()
            out[key + "_b"] = b.numpy()
            out[key + "_cost"] = cost.numpy()
            out[key + "_log_u"] = log_u.numpy()
            out[key + "_log_v"] = log_v.numpy()
            out[key + "_dist"] = solver(src, tgt).detach().numpy()


def pointcloud_cases(out, ref_root):
    """Log-domain iterations of the reference (optimal_transport.py:96-125) on rectangular
    squared-Euclidean costs between point clouds, float64, fixed iteration counts."""
    path = os.path.join(ref_root, "torchmorph", "optimal_transport.py")
    spec = importlib.util.spec_from_file_location("ref_optimal_transport_pc", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    import torch

    rng = np.random.default_rng(77)
    for n, m, eps, iters in [(7, 11, 0.5, 40), (20, 13, 0.1, 60), (5, 5, 0.05, 80)]:
        means = rng.uniform(-1, 1, (4, 3))
        x = means[rng.integers(0, 4, n)] + 0.2 * rng.standard_normal((n, 3))
        y = means[rng.integers(0, 4, m)] + 0.2 * rng.standard_normal((m, 3))
        cost = ((x[:, None] - y[None]) ** 2).sum(-1)
        a = torch.full((1, n), 1.0 / n, dtype=torch.float64)
        b = torch.full((1, m), 1.0 / m, dtype=torch.float64)
        log_u, log_v = mod._log_iterations(a, b, torch.from_numpy(cost), eps, iters, 0.0)
        key = f"pc_{n}x{m}"
        out[key + "_x"] = x
        out[key + "_y"] = y
        out[key + "_eps"] = np.array(eps)
        out[key + "_iters"] = np.array(iters)
        out[key + "_log_u"] = log_u.numpy()[0]
        out[key + "_log_v"] = log_v.numpy()[0]


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    out = {}
    grey_cases(out)
    binary_cases(out)
    distance_cases(out)
    sinkhorn_cases(out, ref_root)
    pointcloud_cases(out, ref_root)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
