"""Child-process runner for the reference's FP64 CUDA library (test infrastructure).

Loads ``oracle/_ref/libmlcpref.so`` (built by ``oracle/ref_build.py``) and
serves calls of its two compute entry points, ``alscpp_``
(src/intertwining.cu:180) and ``intertwinecpp_`` (src/intertwining.cu:98),
with the Fortran host's by-reference argument passing.  It runs in a process
of its own because each entry point ends in ``cudaDeviceReset()``.

Protocol: requests and replies are numpy ``.npz`` archives, each preceded by
its byte length (8-byte little-endian), on the process's original stdin and
stdout.  The library's own printing is sent to stderr.  Every reply carries
``seconds``: the host wall time of the entry-point call, measured after a
``cudaFree(0)`` has created the context, so it covers the reference's whole
call (device allocations, copies, kernels, solves and its closing reset) but
not the context creation that the previous call's reset forces.
"""
from __future__ import annotations

import ctypes
import io
import os
import struct
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libmlcpref.so")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def _read_msg(f):
    hdr = f.read(8)
    if len(hdr) < 8:
        return None
    (n,) = struct.unpack("<Q", hdr)
    data = f.read(n)
    return dict(np.load(io.BytesIO(data), allow_pickle=False))


def _write_msg(f, d):
    buf = io.BytesIO()
    np.savez(buf, **d)
    data = buf.getvalue()
    f.write(struct.pack("<Q", len(data)))
    f.write(data)
    f.flush()


def _dp(a):
    return a.ctypes.data_as(_D)


def _ip(a):
    return a.ctypes.data_as(_I)


def main():
    proto_in = os.fdopen(os.dup(0), "rb")
    proto_out = os.fdopen(os.dup(1), "wb")
    os.dup2(2, 1)  # the library prints with printf/cout: keep it off the protocol
    lib = ctypes.CDLL(LIB, mode=ctypes.RTLD_GLOBAL)
    cudart = ctypes.CDLL("libcudart.so.13")
    cudart.cudaFree.argtypes = [ctypes.c_void_p]
    ri = ctypes.byref
    while True:
        req = _read_msg(proto_in)
        if req is None:
            return 0
        op = str(req["op"])
        if cudart.cudaFree(None) != 0:
            _write_msg(proto_out, {"error": np.array("cudaFree(0) failed: no usable device")})
            continue
        if op == "als":
            # one alscpp_ call per vector: base/coef hold F (rF terms) then G (rG terms)
            coefs = req["coef"].astype(np.float64)
            bases = req["base"].astype(np.float64)
            nbas = np.ascontiguousarray(req["nbas"], dtype=np.int32)
            rF, rG, nals = (int(req[k]) for k in ("rF", "rG", "nals"))
            nv = coefs.shape[0]
            out_c = np.zeros((nv, rF))
            out_b = np.zeros((nv, rF, bases.shape[2]))
            secs = np.zeros(nv)
            for v in range(nv):
                c = np.ascontiguousarray(coefs[v]).copy()
                b = np.ascontiguousarray(bases[v]).copy()
                a = [ctypes.c_int(x) for x in (nbas.size, rF, rG, nals)]
                cudart.cudaFree(None)
                t0 = time.perf_counter()
                lib.alscpp_(_dp(c), _dp(b), _ip(nbas), ri(a[0]), ri(a[1]), ri(a[2]), ri(a[3]))
                secs[v] = time.perf_counter() - t0
                out_c[v] = c[:rF]
                out_b[v] = b[:rF]
            _write_msg(proto_out, {"coef": out_c, "base": out_b, "seconds": secs})
        elif op == "cycle":
            base = np.ascontiguousarray(req["base"], dtype=np.float64).copy()
            coef = np.ascontiguousarray(req["coef"], dtype=np.float64).copy()
            eigv = np.ascontiguousarray(req["eigv"], dtype=np.float64).copy()
            nbas = np.ascontiguousarray(req["nbas"], dtype=np.int32).copy()
            opid = np.ascontiguousarray(req["opid"], dtype=np.int32).copy()
            mptr = np.ascontiguousarray(req["mptr"], dtype=np.int32).copy()
            hcoef = np.ascontiguousarray(req["hcoef"], dtype=np.float64).copy()
            mat = np.ascontiguousarray(req["mat"], dtype=np.float64).copy()
            rk, nbloc, npow, nals, ishift = (int(req[k]) for k in ("rk", "nbloc", "npow", "nals", "ishift"))
            a = [ctypes.c_int(x) for x in (rk, nbas.size, nbloc, opid.size, mptr.size, mat.size, npow, 1, nals,
                                           ishift)]
            upd = ctypes.c_bool(bool(req["update"]))
            esh = ctypes.c_double(float(req["eshift"]))
            t0 = time.perf_counter()
            lib.intertwinecpp_(_dp(base), _dp(coef), _ip(nbas), ri(a[0]), ri(a[1]), ri(a[2]), _ip(opid), _ip(mptr),
                               _dp(hcoef), _dp(mat), ri(a[3]), ri(a[4]), ri(a[5]), _dp(eigv), ri(a[6]), ri(a[7]),
                               ri(a[8]), ri(upd), ri(a[9]), ri(esh))
            secs = time.perf_counter() - t0
            _write_msg(proto_out, {"base": base, "coef": coef, "eigv": eigv, "seconds": np.array(secs)})
        else:
            _write_msg(proto_out, {"error": np.array(f"unknown op {op}")})


if __name__ == "__main__":
    sys.exit(main())
