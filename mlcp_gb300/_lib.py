"""Loader for the C-ABI library ``libmlcp_gb300.so`` (built in-tree).

The product path has no CPU fallback: if the library cannot be built or
loaded, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

_lock = threading.Lock()
_lib = None

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_LL = ctypes.POINTER(ctypes.c_longlong)
_V = ctypes.c_void_p


class MlcpError(RuntimeError):
    """Raised when an entry point of libmlcp_gb300 reports a failure."""


def lib_path() -> str:
    from . import build as _build
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if build_if_missing:
            from . import build as _build
            path = _build.build()
        if not os.path.exists(path):
            raise MlcpError(f"libmlcp_gb300.so not found at {path}; run mlcp_gb300.build.build()")
        L = ctypes.CDLL(path)
        L.mlcp_gb300_last_error.restype = ctypes.c_char_p
        L.mlcp_gb300_last_error.argtypes = []
        L.mlcp_gb300_last_status.restype = ctypes.c_int
        L.mlcp_als_batched.restype = ctypes.c_int
        L.mlcp_als_batched.argtypes = [ctypes.c_int, ctypes.c_int, _I, _I, _I, _LL, _V, _V, ctypes.c_int, _V, _V]
        L.mlcp_als_batched_host.restype = ctypes.c_int
        L.mlcp_als_batched_host.argtypes = [ctypes.c_int, ctypes.c_int, _I, _I, _I, _LL, _D, _D, ctypes.c_int, _V]
        L.mlcp_als_noalloc.restype = ctypes.c_int
        L.mlcp_als_noalloc.argtypes = [ctypes.c_int, _I, ctypes.c_int, ctypes.c_int, _V, _V, ctypes.c_int, _V, _V]
        L.mlcp_cp_dot_batched.restype = ctypes.c_int
        L.mlcp_cp_dot_batched.argtypes = [ctypes.c_int, ctypes.c_int, _I, _LL, _I, _LL, _I, _V, _V, _V, _V]
        L.mlcp_gb300_wait_selftest.restype = ctypes.c_int
        L.mlcp_gb300_wait_selftest.argtypes = [_I]
        L.mlcp_gb300_set_kernel_timing.restype = None
        L.mlcp_gb300_set_kernel_timing.argtypes = [ctypes.c_int]
        L.mlcp_gb300_last_kernel_ms.restype = ctypes.c_double
        L.mlcp_gb300_last_kernel_ms.argtypes = []
        L.alscpp_.restype = None
        L.alscpp_.argtypes = [_D, _D, _I, _I, _I, _I, _I]
        if hasattr(L, "intertwinecpp_"):
            L.intertwinecpp_.restype = None
            L.intertwinecpp_.argtypes = [_D, _D, _I, _I, _I, _I, _I, _I, _D, _D, _I, _I, _I, _D, _I, _I, _I,
                                         ctypes.POINTER(ctypes.c_bool), _I, _D]
        if hasattr(L, "getqhqdiagcpp_"):
            L.getqhqdiagcpp_.restype = None
            L.getqhqdiagcpp_.argtypes = [_D, _D, _I, _I, _I, _I, _I, _I, _I, _D, _D, _I, _I, _I, _D]
        if hasattr(L, "intertwineraggedcpp_"):
            L.intertwineraggedcpp_.restype = None
            L.intertwineraggedcpp_.argtypes = [_D, _D, _I, _I, _I, _I, _I, _I, _I, _D, _D, _I, _I, _I, _D, _I, _I, _I,
                                               ctypes.POINTER(ctypes.c_bool), _I, _D]
        if hasattr(L, "getqhqcpp_"):
            L.getqhqcpp_.restype = None
            L.getqhqcpp_.argtypes = [_D, _D, _I, _I, _I, _I, _I, _I, _D, _D, _I, _I, _I, _D, _V]
        if hasattr(L, "getspectralrangecpp_"):
            L.getspectralrangecpp_.restype = None
            L.getspectralrangecpp_.argtypes = [_D, _D, _I, _I, _I, _I, _I, _I, _I, _D, _D, _I, _I, _I, _D]
        if hasattr(L, "updateopermatcpp_"):
            L.updateopermatcpp_.restype = None
            L.updateopermatcpp_.argtypes = [_I, _D, _D, _I, _I, _I, _I, _I, _D, _D]
        if hasattr(L, "diagonalizecpp_"):
            L.diagonalizecpp_.restype = None
            L.diagonalizecpp_.argtypes = [_D, _D, _I, _I, _I, _I, _I, _I, _D, _D, _I, _I, _I, _D, _I]
        if hasattr(L, "reducsvdcpp_"):
            L.reducsvdcpp_.restype = None
            L.reducsvdcpp_.argtypes = [_D, _D, _I, _I, _I, _I, _D, _D, _D, _I]
        if hasattr(L, "sortvecscpp_"):
            L.sortvecscpp_.restype = None
            L.sortvecscpp_.argtypes = [_D, _D, _I, _I, _I, _I, _D, _I, _D]
        if hasattr(L, "mlcp_save_psi"):
            L.mlcp_save_psi.restype = ctypes.c_int
            L.mlcp_save_psi.argtypes = [ctypes.c_char_p, ctypes.c_int, _D, ctypes.c_int, _D, _D, ctypes.c_int, _I,
                                        _I, _D, _D]
            L.mlcp_read_psi.restype = ctypes.c_int
            L.mlcp_read_psi.argtypes = [ctypes.c_char_p, _I, _D, ctypes.c_int, _D, _D, ctypes.c_int, _I,
                                        ctypes.c_int, _I, _D, _D, _I]
        L.mlcp_gb300_set_autotune.restype = None
        L.mlcp_gb300_set_autotune.argtypes = [ctypes.c_int]
        L.mlcp_gb300_set_als_engine.restype = None
        L.mlcp_gb300_set_als_engine.argtypes = [ctypes.c_int]
        L.mlcp_gb300_als_engine.restype = ctypes.c_int
        L.mlcp_gb300_als_engine.argtypes = []
        L.mlcp_gb300_set_cycle_graph.restype = None
        L.mlcp_gb300_set_cycle_graph.argtypes = [ctypes.c_int]
        L.mlcp_gb300_autotune_report.restype = ctypes.c_int
        L.mlcp_gb300_autotune_report.argtypes = [ctypes.c_char_p, ctypes.c_int]
        _F = ctypes.c_float
        _i = ctypes.c_int
        L.mlcp_mlp_gemm.restype = _i
        L.mlcp_mlp_gemm.argtypes = [_V, _V, _i, _i, _i, _i, _i, _V, _i, _V, _i, _V, _i, _V, _i, _V, _i, _i, _V, _V]
        L.mlcp_mlp_loss.restype = _i
        L.mlcp_mlp_loss.argtypes = [_V, _V, _i, _i, _i, _i, _V, _V, _V, _V]
        L.mlcp_mlp_colsum.restype = _i
        L.mlcp_mlp_colsum.argtypes = [_V, _i, _i, _i, _V, _V]
        L.mlcp_mlp_adam.restype = _i
        L.mlcp_mlp_adam.argtypes = [_V, _V, _V, _V, _i, _i, _F, _F, _F, _F, _i, _V, _V, _V]
        L.mlcp_ws_features.restype = _i
        L.mlcp_ws_features.argtypes = [_i, _i, _i, _i, _V, _V, _i, _V, _V, _V, _i, _V]
        L.mlcp_ws_targets.restype = _i
        L.mlcp_ws_targets.argtypes = [_i, _i, _i, _i, _V, _V, _i, _V, _V, _V, _V, _i, _V]
        L.mlcp_ws_apply.restype = _i
        L.mlcp_ws_apply.argtypes = [_i, _i, _i, _i, _V, _V, _i, _V, _V, _V, _V, _i, _V]
        if hasattr(L, "intwdevicemem_"):
            L.intwdevicemem_.restype = None
            L.intwdevicemem_.argtypes = [_I, _I, _I, _I, _I, _I, _I, ctypes.POINTER(ctypes.c_bool), _I]
        _lib = L
        return L


def check(rc: int) -> None:
    if rc != 0:
        msg = load().mlcp_gb300_last_error().decode(errors="replace")
        raise MlcpError(f"libmlcp_gb300 error {rc}: {msg}")


def last_status() -> int:
    return load().mlcp_gb300_last_status()


def autotune_report() -> str:
    """The autotuner's cached launch shapes and trial times."""
    L = load()
    n = L.mlcp_gb300_autotune_report(None, 0)
    buf = ctypes.create_string_buffer(n + 1)
    L.mlcp_gb300_autotune_report(buf, n + 1)
    return buf.value.decode()


def set_als_engine(engine: int) -> None:
    """Product-pass engine of the batched ALS: 0 automatic (autotuned), 1 CUDA
    cores, 2 tensor cores where the shape fits."""
    load().mlcp_gb300_set_als_engine(int(engine))


def als_engine() -> int:
    return int(load().mlcp_gb300_als_engine())


def last_error() -> str:
    return load().mlcp_gb300_last_error().decode(errors="replace")
