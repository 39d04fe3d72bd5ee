"""Restart of the power-iteration block: the reference's SavePsi / ReadPsi
(src/Restart.f90:579-610 and :733-755), with SavePsiFile / ReadPsiFile
(:759-793 and :614-731); the solver calls them at src/Solver.f90:340, 370
and 432.

The file format is the reference's gfortran unformatted sequential file, so a
restart written by the reference reads here and the other way round.  The
record I/O is native (``mlcp_save_psi`` / ``mlcp_read_psi`` in the C ABI);
this module adds the reference's two-file scheme: every save writes
``<resfile>_1_psi.rst`` and then ``<resfile>_2_psi.rst`` (so that a crash
during one write leaves the other intact), and a read tries the first and then
the second.  ``resfile`` starting with ``none`` disables saving, as in the
reference.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


@dataclass
class PsiState:
    """What a restart file holds: the save counter isavi, the spectral
    bounds, the eigenvalue estimates and their deltas, and the block
    (vector i has ranks[i] terms; coef/base hold the vectors back to back,
    base with nD = sum(nbas) values per term)."""
    isavi: int
    bounds: np.ndarray
    eigv: np.ndarray
    delta: np.ndarray
    nbas: np.ndarray
    ranks: np.ndarray
    coef: np.ndarray
    base: np.ndarray

    def block(self):
        """(base, coef) reshaped as a block of equal-rank vectors:
        base [nev, rk, nD], coef [nev, rk].  Raises if the ranks differ."""
        if self.ranks.size and np.any(self.ranks != self.ranks[0]):
            raise ValueError("vectors of the restart file have different ranks")
        nev, nD = self.eigv.size, int(self.nbas.sum())
        rk = int(self.ranks[0]) if nev else 0
        return self.base.reshape(nev, rk, nD), self.coef.reshape(nev, rk)


def _check(L):
    if L.mlcp_gb300_last_status() != 0:
        raise _lib.MlcpError(_lib.last_error())


def save_psi_file(path: str, isavi: int, bounds, eigv, delta, base, coef, nbas, ranks=None) -> None:
    """SavePsiFile: writes one restart file.  base/coef: a block
    [nev, rk, nD] / [nev, rk], or flat arrays with per-vector ``ranks``."""
    eig = np.ascontiguousarray(eigv, dtype=np.float64).ravel()
    dl = np.ascontiguousarray(delta, dtype=np.float64).ravel()
    bd = np.ascontiguousarray(bounds, dtype=np.float64).ravel()
    nb = np.ascontiguousarray(nbas, dtype=np.int32).ravel()
    nev = eig.size
    if dl.size != nev or bd.size != 2:
        raise ValueError("delta must have nev entries and bounds two")
    cf = np.ascontiguousarray(coef, dtype=np.float64)
    if ranks is None:
        rk = np.full(nev, cf.reshape(nev, -1).shape[1] if nev else 0, dtype=np.int32)
    else:
        rk = np.ascontiguousarray(ranks, dtype=np.int32).ravel()
    cf = cf.ravel()
    bs = np.ascontiguousarray(base, dtype=np.float64).ravel()
    if rk.size != nev or cf.size != int(rk.sum()) or bs.size != cf.size * int(nb.sum()):
        raise ValueError("base/coef do not match ranks and nbas")
    L = _lib.load()
    L.mlcp_save_psi(str(path).encode(), int(isavi), bd.ctypes.data_as(_D), nev, eig.ctypes.data_as(_D),
                    dl.ctypes.data_as(_D), nb.size, nb.ctypes.data_as(_I), rk.ctypes.data_as(_I),
                    cf.ctypes.data_as(_D), bs.ctypes.data_as(_D))
    _check(L)


def read_psi_file(path: str, nev: int, nbas, max_terms: int):
    """ReadPsiFile: returns a PsiState, or None when the file is missing,
    unreadable or does not match nev and nbas (the reference's
    success = .FALSE.).  max_terms bounds the total number of terms."""
    nb = np.ascontiguousarray(nbas, dtype=np.int32).ravel()
    nD = int(nb.sum())
    isavi = ctypes.c_int(0)
    ok = ctypes.c_int(0)
    bd = np.zeros(2)
    eig = np.zeros(nev)
    dl = np.zeros(nev)
    rk = np.zeros(nev, dtype=np.int32)
    cf = np.zeros(max(max_terms, 1))
    bs = np.zeros(max(max_terms, 1) * nD)
    L = _lib.load()
    L.mlcp_read_psi(str(path).encode(), ctypes.byref(isavi), bd.ctypes.data_as(_D), int(nev),
                    eig.ctypes.data_as(_D), dl.ctypes.data_as(_D), nb.size, nb.ctypes.data_as(_I), int(max_terms),
                    rk.ctypes.data_as(_I), cf.ctypes.data_as(_D), bs.ctypes.data_as(_D), ctypes.byref(ok))
    _check(L)
    if not ok.value:
        return None
    terms = int(rk.sum())
    return PsiState(isavi.value, bd, eig, dl, nb.copy(), rk, cf[:terms].copy(), bs[:terms * nD].copy())


def save_psi(resfile: str, isavi: int, bounds, eigv, delta, base, coef, nbas, ranks=None) -> None:
    """SavePsi: writes <resfile>_1_psi.rst, then <resfile>_2_psi.rst; does
    nothing when resfile starts with 'none'."""
    if str(resfile).strip().startswith("none"):
        return
    for k in (1, 2):
        save_psi_file(f"{str(resfile).strip()}_{k}_psi.rst", isavi, bounds, eigv, delta, base, coef, nbas, ranks)


def read_psi(resfile: str, nev: int, nbas, max_terms: int, dorestart: bool = True):
    """ReadPsi: None unless dorestart; else the first of
    <resfile>_1_psi.rst and <resfile>_2_psi.rst that reads and matches."""
    if not dorestart:
        return None
    for k in (1, 2):
        st = read_psi_file(f"{str(resfile).strip()}_{k}_psi.rst", nev, nbas, max_terms)
        if st is not None:
            return st
    return None
