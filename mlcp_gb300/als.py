"""Host-side interface to the explicit-target ALS rank reduction.

Mirrors the reference's ALSCPP/alscpp_ operator (src/GPUIterate.f90:212-285,
src/intertwining.cu:180): a CP vector F of rank rF (terms 0..rF-1, also the
starting guess) is fitted to a target G of rank rG (the following rG terms)
by ``nals`` ALS sweeps; F is overwritten in place.  The batched forms reduce
many independent (F, G) pairs in one launch.

Arrays use the reference layout: ``base`` is (nterms, nD) with row = term,
``coef`` is (nterms,).  Device-resident calls take torch CUDA float64
tensors (PyTorch only supplies memory and streams); host calls take numpy.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_LL = ctypes.POINTER(ctypes.c_longlong)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32))


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64))


_STREAM_LEGACY = 1  # cudaStreamLegacy: the legacy default stream


def _stream_handle(stream) -> int:
    """cudaStream_t for the C ABI.  torch reports its default stream as 0, which
    the library would read as "use the library's own stream"; it is passed as
    cudaStreamLegacy instead so the work is ordered with torch's."""
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    h = stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)
    return h if h != 0 else _STREAM_LEGACY


def reduce_batched(coef, base, nbas: Sequence[int], rF: Sequence[int], rG: Sequence[int],
                   term_off: Sequence[int], nals: int, status=None, stream=None) -> None:
    """Batched ALS on device tensors (torch, float64, CUDA).  Vector v owns
    terms [term_off[v], term_off[v]+rF[v]+rG[v]); its F terms are overwritten.
    Enqueued on ``stream`` (default: torch's current stream)."""
    import torch
    if not (coef.is_cuda and base.is_cuda) or coef.dtype != torch.float64 or base.dtype != torch.float64:
        raise TypeError("coef and base must be float64 CUDA tensors")
    if not (coef.is_contiguous() and base.is_contiguous()):
        raise ValueError("coef and base must be contiguous")
    nb, rf, rg, to = _i32(nbas), _i32(rF), _i32(rG), _i64(term_off)
    st = None
    if status is not None:
        if status.dtype != torch.int32 or not status.is_cuda:
            raise TypeError("status must be an int32 CUDA tensor")
        st = status.data_ptr()
    rc = _lib.load().mlcp_als_batched(len(rf), len(nb), nb.ctypes.data_as(_I), rf.ctypes.data_as(_I),
                                      rg.ctypes.data_as(_I), to.ctypes.data_as(_LL), coef.data_ptr(),
                                      base.data_ptr(), int(nals), st, _stream_handle(stream))
    _lib.check(rc)


def reduce_batched_host(coef: np.ndarray, base: np.ndarray, nbas, rF, rG, term_off, nals: int,
                        stream=None) -> None:
    """Batched ALS on host arrays (in place): host->device copy, reduction and
    device->host copy of the F terms, synchronised before returning when no
    stream is given."""
    if coef.dtype != np.float64 or base.dtype != np.float64:
        raise TypeError("coef and base must be float64")
    if not (coef.flags.c_contiguous and base.flags.c_contiguous):
        raise ValueError("coef and base must be C-contiguous")
    nb, rf, rg, to = _i32(nbas), _i32(rF), _i32(rG), _i64(term_off)
    sh = None if stream is None else _stream_handle(stream)  # None: library stream, synchronised
    rc = _lib.load().mlcp_als_batched_host(len(rf), len(nb), nb.ctypes.data_as(_I), rf.ctypes.data_as(_I),
                                           rg.ctypes.data_as(_I), to.ctypes.data_as(_LL),
                                           coef.ctypes.data_as(_D), base.ctypes.data_as(_D), int(nals), sh)
    _lib.check(rc)


def alscpp(coef: np.ndarray, base: np.ndarray, nbas, rF: int, rG: int, nals: int) -> None:
    """The reference's alscpp_ through the C ABI: in-place on host arrays."""
    nb = _i32(nbas)
    a = [ctypes.c_int(len(nb)), ctypes.c_int(rF), ctypes.c_int(rG), ctypes.c_int(nals)]
    L = _lib.load()
    L.alscpp_(coef.ctypes.data_as(_D), base.ctypes.data_as(_D), nb.ctypes.data_as(_I),
              *[ctypes.byref(x) for x in a])
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())


def cp_dot_batched(coef, base, nbas, x_off, rx, y_off, ry, out, stream=None) -> None:
    """out[v] = <X_v, Y_v> (FP64) for CP vectors stored as term ranges of
    device tensors coef/base (reference layout)."""
    nb, xo, rxa, yo, rya = _i32(nbas), _i64(x_off), _i32(rx), _i64(y_off), _i32(ry)
    rc = _lib.load().mlcp_cp_dot_batched(len(rxa), len(nb), nb.ctypes.data_as(_I), xo.ctypes.data_as(_LL),
                                         rxa.ctypes.data_as(_I), yo.ctypes.data_as(_LL), rya.ctypes.data_as(_I),
                                         coef.data_ptr(), base.data_ptr(), out.data_ptr(), _stream_handle(stream))
    _lib.check(rc)
