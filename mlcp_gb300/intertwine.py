"""Host-side interface to one intertwined power cycle.

Mirrors the reference's IntertwineCPP/intertwinecpp_ operator
(src/GPUIterate.f90:89-187, src/intertwining.cu:98): for a block of nbloc
CP vectors of rank rk and a Hamiltonian operator list, run npow ALS-fitted
applications of (H - Eshift), the ALS-guided Gram-Schmidt, and (update=True)
the block Rayleigh-Ritz problem and ALS-fitted vector updates.  The call
goes through the C ABI with the reference's by-reference argument passing.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def intertwine(base: np.ndarray, coef: np.ndarray, nbas, rk: int, nbloc: int, hl, eigv: np.ndarray, npow: int,
               nals: int, update: bool = True, ishift: int = 1, Eshift: float = 0.0, ncpu: int = 1, ranks=None):
    """Run one cycle on copies of (base, coef, eigv) and return the new
    (base, coef, eigv).  base is (nbloc*rk, nD) with row = term.  With
    ``ranks`` (one per vector, each <= rk) the block is ragged and the cycle
    goes through intertwineraggedcpp_: vector v's terms at or beyond
    ranks[v] are zero-weight padding."""
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    eig = np.ascontiguousarray(eigv, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    opid = np.ascontiguousarray(hl.opid, dtype=np.int32).copy()
    mptr = np.ascontiguousarray(hl.mptr, dtype=np.int32).copy()
    hcoef = np.ascontiguousarray(hl.coef, dtype=np.float64).copy()
    mat = np.ascontiguousarray(hl.mat, dtype=np.float64).copy()
    ints = [ctypes.c_int(x) for x in (rk, nb.size, nbloc, opid.size, mptr.size, mat.size, npow, ncpu, nals,
                                      ishift)]
    upd = ctypes.c_bool(bool(update))
    esh = ctypes.c_double(float(Eshift))
    L = _lib.load()
    if ranks is not None:
        rv = np.ascontiguousarray(ranks, dtype=np.int32).copy()
        if rv.size != nbloc:
            raise ValueError(f"ranks has {rv.size} entries for a block of {nbloc}")
        L.intertwineraggedcpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I),
                               ctypes.byref(ints[0]), rv.ctypes.data_as(_I), ctypes.byref(ints[1]),
                               ctypes.byref(ints[2]), opid.ctypes.data_as(_I), mptr.ctypes.data_as(_I),
                               hcoef.ctypes.data_as(_D), mat.ctypes.data_as(_D), ctypes.byref(ints[3]),
                               ctypes.byref(ints[4]), ctypes.byref(ints[5]), eig.ctypes.data_as(_D),
                               ctypes.byref(ints[6]), ctypes.byref(ints[7]), ctypes.byref(ints[8]), ctypes.byref(upd),
                               ctypes.byref(ints[9]), ctypes.byref(esh))
        if L.mlcp_gb300_last_status() != 0:
            raise _lib.MlcpError(_lib.last_error())
        return base, coef, eig
    L.intertwinecpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I),
                     ctypes.byref(ints[0]), ctypes.byref(ints[1]), ctypes.byref(ints[2]),
                     opid.ctypes.data_as(_I), mptr.ctypes.data_as(_I), hcoef.ctypes.data_as(_D),
                     mat.ctypes.data_as(_D), ctypes.byref(ints[3]), ctypes.byref(ints[4]), ctypes.byref(ints[5]),
                     eig.ctypes.data_as(_D), ctypes.byref(ints[6]), ctypes.byref(ints[7]), ctypes.byref(ints[8]),
                     ctypes.byref(upd), ctypes.byref(ints[9]), ctypes.byref(esh))
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return base, coef, eig


def qhq_diag(base: np.ndarray, coef: np.ndarray, nbas, rk: int, nbloc: int, hl, nconv: int = 0,
             qhqd: np.ndarray | None = None) -> np.ndarray:
    """Reference GetQHQdiag (src/BlockUtils.f90:385-408) through
    getqhqdiagcpp_: Rayleigh quotients <Q_i|H|Q_i>/<Q_i|Q_i> of vectors
    nconv..nbloc-1 (H applied exactly, FP64 on the GPU).  Returns a copy of
    qhqd (zeros when None) with those entries filled."""
    base = np.ascontiguousarray(base, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    out = np.zeros(nbloc) if qhqd is None else np.ascontiguousarray(qhqd, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    opid = np.ascontiguousarray(hl.opid, dtype=np.int32).copy()
    mptr = np.ascontiguousarray(hl.mptr, dtype=np.int32).copy()
    hcoef = np.ascontiguousarray(hl.coef, dtype=np.float64).copy()
    mat = np.ascontiguousarray(hl.mat, dtype=np.float64).copy()
    ints = [ctypes.c_int(x) for x in (rk, nb.size, nbloc, nconv, opid.size, mptr.size, mat.size)]
    L = _lib.load()
    L.getqhqdiagcpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I),
                     *[ctypes.byref(x) for x in ints[:4]], opid.ctypes.data_as(_I), mptr.ctypes.data_as(_I),
                     hcoef.ctypes.data_as(_D), mat.ctypes.data_as(_D), *[ctypes.byref(x) for x in ints[4:]],
                     out.ctypes.data_as(_D))
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return out


def spectral_range(base: np.ndarray, coef: np.ndarray, nbas, rk: int, hl, npow: int, ncyc: int):
    """Reference GetSpectralRange (src/Solver.f90:563-654) through
    getspectralrangecpp_, from the two starting vectors of rank rk in
    (base, coef) -- for two modes the rank-1 starts padded with zero-weight
    terms, which the SVD power recursion fills up to rank rk.  Returns
    (base, coef, bounds) on copies, bounds padded by 0.1 % of the range on
    each side."""
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    opid = np.ascontiguousarray(hl.opid, dtype=np.int32).copy()
    mptr = np.ascontiguousarray(hl.mptr, dtype=np.int32).copy()
    hcoef = np.ascontiguousarray(hl.coef, dtype=np.float64).copy()
    mat = np.ascontiguousarray(hl.mat, dtype=np.float64).copy()
    bounds = np.zeros(2)
    ints = [ctypes.c_int(x) for x in (rk, nb.size, npow, ncyc, opid.size, mptr.size, mat.size)]
    L = _lib.load()
    L.getspectralrangecpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I),
                           *[ctypes.byref(x) for x in ints[:4]], opid.ctypes.data_as(_I), mptr.ctypes.data_as(_I),
                           hcoef.ctypes.data_as(_D), mat.ctypes.data_as(_D), *[ctypes.byref(x) for x in ints[4:]],
                           bounds.ctypes.data_as(_D))
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return base, coef, bounds


def diagonalize(base: np.ndarray, coef: np.ndarray, nbas, rk: int, nbloc: int, hl, nals: int):
    """Reference Diagonalize with intw = .FALSE. (src/BlockUtils.f90:184-225)
    through diagonalizecpp_ on copies: the exact block Rayleigh-Ritz problem
    and the reduced eigenvector combinations.  Returns (base, coef, eigv)."""
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    opid = np.ascontiguousarray(hl.opid, dtype=np.int32).copy()
    mptr = np.ascontiguousarray(hl.mptr, dtype=np.int32).copy()
    hcoef = np.ascontiguousarray(hl.coef, dtype=np.float64).copy()
    mat = np.ascontiguousarray(hl.mat, dtype=np.float64).copy()
    eigv = np.zeros(nbloc)
    ints = [ctypes.c_int(x) for x in (rk, nb.size, nbloc, opid.size, mptr.size, mat.size, nals)]
    L = _lib.load()
    L.diagonalizecpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I),
                      *[ctypes.byref(x) for x in ints[:3]], opid.ctypes.data_as(_I), mptr.ctypes.data_as(_I),
                      hcoef.ctypes.data_as(_D), mat.ctypes.data_as(_D), *[ctypes.byref(x) for x in ints[3:6]],
                      eigv.ctypes.data_as(_D), ctypes.byref(ints[6]))
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return base, coef, eigv


def qhq(base: np.ndarray, coef: np.ndarray, nbas, rk: int, nbloc: int, hl, overlaps: bool = False):
    """Reference GetQHQ / GetOverlaps (src/BlockUtils.f90:229-264, :347-381)
    through getqhqcpp_: the full nbloc x nbloc matrix <Q_j|H|Q_i> (FP64, H
    applied exactly) and, with overlaps, <Q_j|Q_i>."""
    base = np.ascontiguousarray(base, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    opid = np.ascontiguousarray(hl.opid, dtype=np.int32).copy()
    mptr = np.ascontiguousarray(hl.mptr, dtype=np.int32).copy()
    hcoef = np.ascontiguousarray(hl.coef, dtype=np.float64).copy()
    mat = np.ascontiguousarray(hl.mat, dtype=np.float64).copy()
    A = np.zeros((nbloc, nbloc))
    S = np.zeros((nbloc, nbloc)) if overlaps else None
    ints = [ctypes.c_int(x) for x in (rk, nb.size, nbloc, opid.size, mptr.size, mat.size)]
    L = _lib.load()
    L.getqhqcpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I), ctypes.byref(ints[0]),
                 ctypes.byref(ints[1]), ctypes.byref(ints[2]), opid.ctypes.data_as(_I), mptr.ctypes.data_as(_I),
                 hcoef.ctypes.data_as(_D), mat.ctypes.data_as(_D), ctypes.byref(ints[3]), ctypes.byref(ints[4]),
                 ctypes.byref(ints[5]), A.ctypes.data_as(_D), S.ctypes.data_as(_D) if S is not None else None)
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return (A.T.copy(), S.T.copy()) if overlaps else A.T.copy()


def update_opermat(imode: int, base: np.ndarray, coef: np.ndarray, nbas, rk: int, nbloc: int,
                   xmats: np.ndarray) -> np.ndarray:
    """Reference UpdateOperMat (src/Updater.f90:110-151) through
    updateopermatcpp_ for the operators xmats (one packed upper triangle per
    row) of mode imode (1-based): returns the packed nbloc x nbloc matrices
    <Q_j, X Q_i>, one row per operator."""
    base = np.ascontiguousarray(base, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    xm = np.ascontiguousarray(np.atleast_2d(xmats), dtype=np.float64)
    out = np.zeros((xm.shape[0], nbloc * (nbloc + 1) // 2))
    ints = [ctypes.c_int(x) for x in (imode, rk, nb.size, nbloc, xm.shape[0])]
    L = _lib.load()
    L.updateopermatcpp_(ctypes.byref(ints[0]), base.ctypes.data_as(_D), coef.ctypes.data_as(_D),
                        nb.ctypes.data_as(_I), *[ctypes.byref(x) for x in ints[1:]], xm.ctypes.data_as(_D),
                        out.ctypes.data_as(_D))
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return out


def reduc_svd(base: np.ndarray, coef: np.ndarray, nbas, rG: int, rF: int, redtol: float = 1.0e-12):
    """Reference reduc_SVDa/b (src/REDUCTIONML.f90:296-392) through
    reducsvdcpp_ for a batch of two-mode vectors of rG terms each
    (base [nvec * rG, nD], coef [nvec * rG]).  Returns (base [nvec, rF, nD],
    coef [nvec, rF], rank [nvec]); terms past rank[v] are zero."""
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    if nb.size != 2:
        raise ValueError("reduc_svd reduces two-mode vectors")
    nD = int(nb.sum())
    base = np.ascontiguousarray(base, dtype=np.float64).reshape(-1, rG, nD)
    coef = np.ascontiguousarray(coef, dtype=np.float64).reshape(-1, rG)
    nvec = base.shape[0]
    obase = np.zeros((nvec, rF, nD))
    ocoef = np.zeros((nvec, rF))
    orank = np.zeros(nvec, dtype=np.int32)
    ints = [ctypes.c_int(x) for x in (rG, nvec, rF)]
    tol = ctypes.c_double(float(redtol))
    L = _lib.load()
    L.reducsvdcpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I),
                   *[ctypes.byref(x) for x in ints], ctypes.byref(tol), obase.ctypes.data_as(_D),
                   ocoef.ctypes.data_as(_D), orank.ctypes.data_as(_I))
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return obase, ocoef, orank


def sort_vecs(base: np.ndarray, coef: np.ndarray, nbas, rk: int, eigv: np.ndarray, nconv: int, eref: float):
    """Reference SortVecs (src/BlockUtils.f90:520-583) through sortvecscpp_
    on copies; returns (base, coef, eigv, nconv)."""
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    eig = np.ascontiguousarray(eigv, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32).copy()
    ints = [ctypes.c_int(x) for x in (rk, nb.size, eig.size, nconv)]
    e = ctypes.c_double(float(eref))
    L = _lib.load()
    L.sortvecscpp_(base.ctypes.data_as(_D), coef.ctypes.data_as(_D), nb.ctypes.data_as(_I),
                   *[ctypes.byref(x) for x in ints[:3]], eig.ctypes.data_as(_D), ctypes.byref(ints[3]),
                   ctypes.byref(e))
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())
    return base, coef, eig, ints[3].value


def block_shift(eigv, emax: float) -> float:
    """Reference GetBlockShift (src/BlockPower.f90:20-45): half way between an
    estimate of the first eigenvalue above the block and the spectrum's top."""
    eigv = np.asarray(eigv, dtype=np.float64)
    if eigv.size > 1:
        a = 2 * eigv[-1] - eigv[-2]
    else:
        a = 2 * eigv[0]
    return 0.5 * (a + emax)
