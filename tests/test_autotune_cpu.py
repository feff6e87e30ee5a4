"""Autotuner host logic: the C variant table, work classes and the JSON cache (no GPU)."""

import json

import pytest

from torchmorph_gb300 import _lib, autotune


@pytest.fixture(autouse=True)
def _restore_table():
    yield
    for op in autotune.OPS:
        for cls in range(64):
            autotune.set_variant(op, cls, -1)


def test_variant_table_and_validation():
    lib = _lib.load()
    assert [autotune.variants(op) for op in ("grey_flat2d", "sinkhorn_f32", "edt_3d", "cdt_3d")] == [4, 4, 2, 3]
    assert autotune.get_variant("edt_3d", 23) == -1
    autotune.set_variant("edt_3d", 23, 1)
    assert autotune.get_variant("edt_3d", 23) == 1
    assert autotune.get_variant("cdt_3d", 23) == -1  # per operator
    assert lib.tm_tune_set(2, 23, 2) == 1 and "variants 0..1" in lib.tm_last_error().decode()
    assert lib.tm_tune_set(9, 0, 0) == 1
    assert lib.tm_tune_set(0, 64, 0) == 1
    assert lib.tm_tune_get(9, 0) == -1


def test_work_classes():
    assert autotune.work_class("edt_3d", 4 * 128 ** 3) == 23
    assert autotune.work_class("grey_flat2d", 1) == 0
    assert autotune.work_class("grey_flat2d", 2 ** 62) == 62
    # Sinkhorn: 8 * min(7, log2 n) + min(7, log2 d - 6)
    assert autotune.work_class("sinkhorn_f32", 256, 8192) == 8 * 7 + 7
    assert autotune.work_class("sinkhorn_f32", 5, 96) == 8 * 2 + 0
    assert autotune.work_class("sinkhorn_f32", 1, 1) == 0


def test_cache_round_trip_and_apply(tmp_path):
    path = str(tmp_path / "t.json")
    assert autotune.load_cache(path) == {"version": 1, "devices": {}}
    data = autotune.load_cache(path)
    data["devices"]["GPU A"] = {"edt_3d": {"23": 1}, "sinkhorn_f32": {"63": 3, "2": 9},
                                "unknown_op": {"1": 0}, "cdt_3d": {"x": 1, "4": 3}}
    autotune.save_cache(data, path)
    with open(path) as f:
        assert json.load(f)["devices"]["GPU A"]["edt_3d"] == {"23": 1}
    assert autotune.apply_cache("GPU B", path) == 0
    assert autotune.apply_cache("GPU A", path) == 2  # the out-of-range and malformed entries are skipped
    assert autotune.get_variant("edt_3d", 23) == 1
    assert autotune.get_variant("sinkhorn_f32", 63) == 3
    assert autotune.get_variant("sinkhorn_f32", 2) == -1
    with open(path, "w") as f:
        f.write("{not json")
    assert autotune.load_cache(path)["devices"] == {}
    with pytest.raises(ValueError, match="unknown operator"):
        autotune.tune("nope", lambda: None, 1)
