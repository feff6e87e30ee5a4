"""The C-ABI library loads, exports every declared symbol, and rejects bad
arguments on the host (no GPU work is started by these calls)."""

import ctypes
import glob
import os
import re

import pytest

from torchmorph_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(tm_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_declarations():
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_status_strings_and_version():
    lib = _lib.load()
    assert lib.tm_status_string(0) == b"ok"
    assert lib.tm_status_string(1) == b"invalid argument"
    assert lib.tm_version() >= 100


def _err(status):
    return status, _lib.load().tm_last_error().decode()


def test_rejects_bad_geometry_without_touching_the_device():
    lib = _lib.load()
    shape = _lib.i64_array([4, 4])
    st = _lib.f32_array([0.0] * 9)
    fp = (ctypes.c_uint8 * 9)(*([1] * 9))
    ss = _lib.i64_array([3, 3])
    org = _lib.i64_array([0, 0])
    s, msg = _err(lib.tm_grey_erosion(None, None, 1, 0, shape, ctypes.cast(st, _lib.F32P),
                                      ctypes.cast(fp, _lib.U8P), ss, org, 1, 0.0, None))
    assert s == 1 and "ndim" in msg
    s, msg = _err(lib.tm_grey_erosion(None, None, 1, 2, shape, ctypes.cast(st, _lib.F32P),
                                      ctypes.cast(fp, _lib.U8P), ss, org, 1, 0.0, None))
    assert s == 1 and "NULL" in msg
    bad = _lib.i64_array([4, 0])
    s, msg = _err(lib.tm_edt(ctypes.c_void_p(16), 0, 1, 2, bad, None, None, None, None, None, 0, None))
    assert s == 1 and "sizes must be >= 1" in msg
    s, msg = _err(lib.tm_edt(ctypes.c_void_p(16), 7, 1, 2, shape, None, ctypes.c_void_p(16), None,
                             None, None, 0, None))
    assert s == 1 and "dtype" in msg
    s, msg = _err(lib.tm_edt(ctypes.c_void_p(16), 0, 1, 2, shape, None, None, None, None, None, 0,
                             None))
    assert s == 1 and "output" in msg
    big = _lib.i64_array([40000, 40000])
    s, msg = _err(lib.tm_edt(ctypes.c_void_p(16), 0, 1, 2, big, None, ctypes.c_void_p(16), None,
                             None, None, 0, None))
    assert s == 4
    s, msg = _err(lib.tm_cdt(ctypes.c_void_p(16), 0, 1, 2, shape, 5, ctypes.c_void_p(16), None,
                             None, 0, None))
    assert s == 1 and "metric" in msg
    need = lib.tm_cdt_workspace_size(1, 2, shape)
    assert need > 0
    s, msg = _err(lib.tm_cdt(ctypes.c_void_p(16), 0, 1, 2, shape, 0, ctypes.c_void_p(16), None,
                             None, 0, None))
    assert s == 5 and "workspace" in msg
    s, msg = _err(lib.tm_sinkhorn_logiter(None, None, None, None, None, None, 1, 4, 1, 1.0, None, 0,
                                          None))
    assert s == 1
    p = ctypes.c_void_p(256)
    s, msg = _err(lib.tm_sinkhorn_fastiter(p, p, p, p, p, p, 2, 4, 3, None, 0, None))
    assert s == 5 and "workspace" in msg
    s, msg = _err(lib.tm_sinkhorn_f32_solve(p, p, p, 2, 4, 0.0, 0, 10, 0.0, 1, p, p, None, None, None,
                                            None, 0, None))
    assert s == 1 and "epsilon" in msg
    s, msg = _err(lib.tm_sinkhorn_f32_solve(p, p, p, 2, 4, 0.1, 0, 10, 0.0, 1, p, p, None, None, None,
                                            None, 0, None))
    assert s == 5 and "workspace" in msg
    s, msg = _err(lib.tm_sinkhorn_plan(p, p, p, 0, 4, 0.1, p, None))
    assert s == 1 and "n >= 1" in msg


def test_workspace_sizes():
    lib = _lib.load()
    assert lib.tm_sinkhorn_iter_workspace_size() == 256
    w = lib.tm_sinkhorn_f32_workspace_size(3, 300, 0, 100, 10, 0)
    assert w >= 2 * 300 * 300 * 4 + 2 * 3 * 300 * 4
    assert lib.tm_sinkhorn_f32_workspace_size(3, 300, 1, 100, 10, 0) < w  # the log form keeps no K
    # the line cost |i - j| is computed in the kernels: no (d, d) matrix in the workspace
    assert lib.tm_sinkhorn_f32_workspace_size(3, 300, 0, 100, 10, 1) < 300 * 300 * 4
    assert lib.tm_sinkhorn_f32_workspace_size(3, 300, 1, 100, 10, 1) < 300 * 300 * 4
    assert lib.tm_edt_workspace_size(1, 1, _lib.i64_array([10]), None) == 0
    n2 = lib.tm_edt_workspace_size(4, 3, _lib.i64_array([8, 8, 8]), None)
    assert n2 >= 4 * 512 * (2 + 4)
    n3 = lib.tm_edt_workspace_size(4, 3, _lib.i64_array([8, 8, 8]), _lib.f32_array([1.0, 1.0, 2.5]))
    assert n3 >= 2 * 2 * 4 * 512 * 4
    assert lib.tm_bfdt_workspace_size(2, 2, _lib.i64_array([5, 5])) >= 2 * 25 * 4


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(ImportError, match="no CPU fallback"):
        _lib.load()
