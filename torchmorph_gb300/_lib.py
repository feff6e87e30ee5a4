"""ctypes binding of libtmcore.so, the C-ABI CUDA library (include/torchmorph_gb300.h).

The library is loaded once per process.  There is no fallback: if the shared
object is missing or fails to load, every operator raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtmcore.so")

_lib = None
_lock = threading.Lock()

c_i64 = ctypes.c_int64
c_int = ctypes.c_int
c_void = ctypes.c_void_p
c_size = ctypes.c_size_t
c_float = ctypes.c_float
c_double = ctypes.c_double
I64P = ctypes.POINTER(ctypes.c_int64)
F32P = ctypes.POINTER(ctypes.c_float)
U8P = ctypes.POINTER(ctypes.c_uint8)

# name -> (restype, argtypes); mirrors include/torchmorph_gb300.h
SIGNATURES = {
    "tm_status_string": (ctypes.c_char_p, [c_int]),
    "tm_last_error": (ctypes.c_char_p, []),
    "tm_version": (c_int, []),
    "tm_device_error": (c_int, [c_int]),
    "tm_grey_erosion": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int,
                                c_float, c_void]),
    "tm_grey_dilation": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int,
                                 c_float, c_void]),
    "tm_binary_erosion": (c_int, [c_void, c_void, c_i64, c_int, I64P, U8P, I64P, I64P, c_int,
                                  c_void]),
    "tm_binary_dilation": (c_int, [c_void, c_void, c_i64, c_int, I64P, U8P, I64P, I64P, c_int,
                                   c_void]),
    "tm_binary_opening": (c_int, [c_void, c_void, c_i64, c_int, I64P, U8P, I64P, I64P, c_int,
                                  c_void]),
    "tm_binary_closing": (c_int, [c_void, c_void, c_i64, c_int, I64P, U8P, I64P, I64P, c_int,
                                  c_void]),
    "tm_edt_workspace_size": (c_size, [c_i64, c_int, I64P, F32P]),
    "tm_edt": (c_int, [c_void, c_int, c_i64, c_int, I64P, F32P, c_void, c_void, c_void, c_void,
                       c_size, c_void]),
    "tm_edt_noalloc": (c_int, [c_void, c_int, c_i64, c_int, I64P, c_void, c_void, c_void, c_void]),
    "tm_cdt_workspace_size": (c_size, [c_i64, c_int, I64P]),
    "tm_cdt": (c_int, [c_void, c_int, c_i64, c_int, I64P, c_int, c_void, c_void, c_void, c_size,
                       c_void]),
    "tm_bfdt_workspace_size": (c_size, [c_i64, c_int, I64P]),
    "tm_bfdt": (c_int, [c_void, c_int, c_i64, c_int, I64P, c_int, F32P, c_void, c_void, c_void,
                        c_size, c_void]),
    "tm_set_grid_wait_budget": (None, [c_i64]),
    "tm_tune_variants": (c_int, [c_int]),
    "tm_tune_class": (c_int, [c_int, c_i64, c_i64]),
    "tm_tune_set": (c_int, [c_int, c_int, c_int]),
    "tm_tune_get": (c_int, [c_int, c_int]),
    "tm_sinkhorn_iter_workspace_size": (c_size, []),
    "tm_sinkhorn_fastiter": (c_int, [c_void, c_void, c_void, c_void, c_void, c_void, c_i64, c_i64,
                                     c_i64, c_void, c_size, c_void]),
    "tm_sinkhorn_logiter": (c_int, [c_void, c_void, c_void, c_void, c_void, c_void, c_i64, c_i64,
                                    c_i64, c_double, c_void, c_size, c_void]),
    "tm_sinkhorn_f32_workspace_size": (c_size, [c_i64, c_i64, c_int, c_i64, c_i64, c_int]),
    "tm_sinkhorn_f32_solve": (c_int, [c_void, c_void, c_void, c_i64, c_i64, c_double, c_int, c_i64,
                                      c_double, c_i64, c_void, c_void, c_void, c_void, c_void, c_void,
                                      c_size, c_void]),
    "tm_sinkhorn_plan": (c_int, [c_void, c_void, c_void, c_i64, c_i64, c_double, c_void, c_void]),
    "tm_sinkhorn_cost_grad": (c_int, [c_void, c_void, c_void, c_void, c_i64, c_i64, c_double, c_void,
                                      c_void]),
    "tm_gemm_bf16x3": (c_int, [c_void, c_void, c_void, c_void, c_void, c_i64, c_i64, c_i64,
                               c_void]),
    "tm_sinkhorn_tc_workspace_size": (c_size, [c_i64, c_i64]),
    "tm_sinkhorn_tc_init": (c_int, [c_void, c_void, c_void, c_i64, c_i64, c_double, c_void, c_size,
                                    c_void]),
    "tm_sinkhorn_tc_iterate": (c_int, [c_i64, c_i64, c_i64, c_void, c_void, c_size, c_void]),
    "tm_sinkhorn_tc_finish": (c_int, [c_i64, c_i64, c_void, c_void, c_void, c_void, c_void, c_size,
                                      c_void]),
    "tm_grey_erosion_arg": (c_int, [c_void, c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P,
                                    c_int, c_float, c_void]),
    "tm_grey_dilation_arg": (c_int, [c_void, c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P,
                                     I64P, c_int, c_float, c_void]),
    "tm_grey_erosion_backward": (c_int, [c_void, c_void, c_void, c_i64, c_int, I64P, U8P, I64P, I64P,
                                         c_int, c_void]),
    "tm_grey_gradient": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int, c_float,
                                 c_void]),
    "tm_grey_laplace": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int, c_float,
                                c_void]),
    "tm_grey_opening": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int, c_float,
                                c_void]),
    "tm_grey_closing": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int, c_float,
                                c_void]),
    "tm_white_tophat": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int, c_float,
                                c_void]),
    "tm_black_tophat": (c_int, [c_void, c_void, c_i64, c_int, I64P, F32P, U8P, I64P, I64P, c_int, c_float,
                                c_void]),
    "tm_grey_dilation_backward": (c_int, [c_void, c_void, c_void, c_i64, c_int, I64P, U8P, I64P, I64P,
                                          c_int, c_void]),
    "tm_pointcloud_sinkhorn_workspace_size": (c_size, [c_i64, I64P, I64P, c_i64]),
    "tm_pointcloud_sinkhorn": (c_int, [c_void, c_void, c_void, c_void, c_i64, I64P, I64P, c_double,
                                       c_i64, c_double, c_i64, c_void, c_void, c_void, c_void, c_void,
                                       c_size, c_void]),
    "tm_pointcloud_sinkhorn_grad_workspace_size": (c_size, [c_i64]),
    "tm_pointcloud_sinkhorn_grad": (c_int, [c_void, c_void, c_void, c_void, c_void, c_void, c_i64, I64P,
                                            I64P, c_double, c_void, c_void, c_void, c_void, c_size,
                                            c_void]),
    "tm_ragged3d_plan_size": (c_size, [c_i64]),
    "tm_ragged3d_plan": (c_int, [c_i64, I64P, I64P, I64P, I64P, c_void, c_size, c_void]),
    "tm_ragged3d_grey_erosion": (c_int, [c_void, c_void, c_void, c_size, c_i64, F32P, U8P, I64P, I64P,
                                         c_int, c_float, c_void]),
    "tm_ragged3d_grey_dilation": (c_int, [c_void, c_void, c_void, c_size, c_i64, F32P, U8P, I64P, I64P,
                                          c_int, c_float, c_void]),
    "tm_ragged3d_binary_erosion": (c_int, [c_void, c_void, c_void, c_size, c_i64, U8P, I64P, I64P, c_int,
                                           c_void]),
    "tm_ragged3d_binary_dilation": (c_int, [c_void, c_void, c_void, c_size, c_i64, U8P, I64P, I64P, c_int,
                                            c_void]),
    "tm_ragged_edt_plan_size": (c_size, [c_i64]),
    "tm_ragged_edt_plan": (c_int, [c_i64, c_int, I64P, I64P, c_void, c_size, c_void]),
    "tm_ragged_edt_workspace_size": (c_size, [c_i64, c_i64]),
    "tm_ragged_edt": (c_int, [c_void, c_int, c_void, c_size, c_i64, c_int, c_i64, c_i64, I64P, c_void, c_void,
                              c_void, c_void, c_size, c_void]),
    "tm_ragged_plan_size": (c_size, [c_i64]),
    "tm_ragged_plan": (c_int, [c_i64, I64P, I64P, I64P, c_void, c_size, c_void]),
    "tm_ragged_grey_erosion": (c_int, [c_void, c_void, c_void, c_size, c_i64, F32P, U8P, I64P, I64P,
                                       c_int, c_float, c_void]),
    "tm_ragged_grey_dilation": (c_int, [c_void, c_void, c_void, c_size, c_i64, F32P, U8P, I64P, I64P,
                                        c_int, c_float, c_void]),
    "tm_ragged_binary_erosion": (c_int, [c_void, c_void, c_void, c_size, c_i64, U8P, I64P, I64P, c_int,
                                         c_void]),
    "tm_ragged_binary_dilation": (c_int, [c_void, c_void, c_void, c_size, c_i64, U8P, I64P, I64P, c_int,
                                          c_void]),
    "tm_ragged_binary_opening": (c_int, [c_void, c_void, c_void, c_size, c_i64, U8P, I64P, I64P, c_int,
                                         c_void]),
    "tm_ragged_binary_closing": (c_int, [c_void, c_void, c_void, c_size, c_i64, U8P, I64P, I64P, c_int,
                                         c_void]),
}

TM_F32 = 0
TM_U8 = 1


class TorchmorphError(RuntimeError):
    """A libtmcore call returned a non-zero tm_status."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def load():
    """Load libtmcore.so (building nothing) and bind every declared symbol."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"torchmorph_gb300: CUDA library {LIB_PATH} is missing; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)"
            )
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    # install the autotuner's cached choices for this device (a missing or bad
    # cache leaves the built-in choices)
    try:
        from . import autotune

        autotune.apply_cache()
    except Exception:  # noqa: BLE001 -- tuning is an optimisation, never a failure
        pass
    return _lib


def available_symbols():
    lib = load()
    return [name for name in SIGNATURES if hasattr(lib, name)]


def check(status: int, what: str) -> None:
    if status != 0:
        lib = load()
        msg = lib.tm_last_error().decode(errors="replace")
        kind = lib.tm_status_string(status).decode(errors="replace")
        raise TorchmorphError(status, f"{what}: {kind}: {msg}")


def i64_array(values):
    values = [int(v) for v in values]
    return (ctypes.c_int64 * max(1, len(values)))(*values)


def f32_array(values):
    values = [float(v) for v in values]
    return (ctypes.c_float * max(1, len(values)))(*values)


def ctypes_f32(t: torch.Tensor):
    """float* view of a contiguous float32 CPU tensor (kept alive by the caller)."""
    return ctypes.cast(t.data_ptr(), F32P)


def ctypes_u8(t: torch.Tensor):
    """uint8* view of a contiguous bool/uint8 CPU tensor (kept alive by the caller)."""
    return ctypes.cast(t.data_ptr(), U8P)


def ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_of(device: torch.device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
