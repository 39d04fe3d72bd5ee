"""The block eigensolver loop around the GPU power cycle: the reference's
SolveHPsi (src/Solver.f90:307-445) for its GPU intertwining solver (styp = -2,
update on; Iterate, :449-559), driven from the host as the Fortran host does:

* the spectral range once (getspectralrangecpp_, from the starting vectors
  of GetSpectralRange, src/Solver.f90:583-606, built here as the reference
  builds them);
* per cycle the block shift of GetBlockShift (src/BlockPower.f90:20-45) and
  one intertwined cycle (intertwinecpp_), then the relative eigenvalue
  changes and their rms, which ends the loop below solvtol; optionally the
  restart files of SavePsi after every cycle.

The starting block is the nev lowest product functions (by total quanta),
each a rank-1 vector raised to rank rk by AugmentVWithRandom's rule
(src/MODVECVECML.f90:1378-1401): seeded random factors normalised per mode,
weight 1e-12 of the smallest weight.
"""
from __future__ import annotations

import itertools

import numpy as np

from . import intertwine as IT


def spectral_start(nbas, rk: int, seed: int = 0):
    """The two starting vectors of GetSpectralRange (src/Solver.f90:583-606):
    the first (lower guess) and last (upper guess) basis function of every
    mode, 1e-15 elsewhere, weight 1; with more than two modes and rk > 1 the
    same rk - 1 seeded random terms (normalised per mode) of weight 1e-7.
    Two modes keep rank 1, padded to rk with zero weights."""
    nbas = np.asarray(nbas, dtype=np.int64)
    nD, D = int(nbas.sum()), nbas.size
    offs = np.concatenate([[0], np.cumsum(nbas)])
    rng = np.random.default_rng(seed)
    rand = rng.uniform(-0.5, 0.5, size=(max(rk - 1, 0), nD))
    for d in range(D):
        blk = rand[:, offs[d]:offs[d + 1]]
        blk /= np.linalg.norm(blk, axis=1, keepdims=True)
    base = np.full((2 * rk, nD), 1e-15)
    coef = np.zeros(2 * rk)
    for j in range(2):
        coef[j * rk] = 1.0
        for d in range(D):
            base[j * rk, offs[d] if j == 0 else offs[d + 1] - 1] = 1.0
        if D > 2 and rk > 1:
            base[j * rk + 1:(j + 1) * rk] = rand
            coef[j * rk + 1:(j + 1) * rk] = 1e-7
    return base, coef


def _with_quanta(nbas, q, prefix=()):
    """Index tuples over the modes with total q, in lexicographic order."""
    d = len(prefix)
    if d == len(nbas):
        if q == 0:
            yield prefix
        return
    rest = sum(n - 1 for n in nbas[d + 1:])
    for i in range(max(0, q - rest), min(q, nbas[d] - 1) + 1):
        yield from _with_quanta(nbas, q - i, prefix + (i,))


def _lowest_products(nbas, nev):
    """The nev product states of lowest total quanta (ties lexicographic),
    generated shell by shell rather than from the whole product space."""
    out = []
    for q in itertools.count():
        if q > sum(n - 1 for n in nbas):
            break
        for st in _with_quanta(nbas, q):
            out.append(st)
            if len(out) == nev:
                return out
    return out


def product_guess(nbas, nev: int, rk: int, seed: int = 0):
    """nev product functions of lowest total quanta (ties in lexicographic
    order) as rank-rk vectors: the product term with weight 1, then rk - 1
    seeded random terms, normalised per mode, of weight 1e-12."""
    nbas = [int(n) for n in nbas]
    offs = np.concatenate([[0], np.cumsum(nbas)])
    nD = int(offs[-1])
    states = _lowest_products(nbas, nev)
    rng = np.random.default_rng(seed)
    base = np.zeros((nev * rk, nD))
    coef = np.zeros(nev * rk)
    for i, st in enumerate(states):
        for d, q in enumerate(st):
            base[i * rk, offs[d] + q] = 1.0
        coef[i * rk] = 1.0
        if rk > 1:
            r = rng.uniform(-0.5, 0.5, size=(rk - 1, nD))
            for d in range(len(nbas)):
                r[:, offs[d]:offs[d + 1]] /= np.linalg.norm(r[:, offs[d]:offs[d + 1]], axis=1, keepdims=True)
            base[i * rk + 1:(i + 1) * rk] = r
            coef[i * rk + 1:(i + 1) * rk] = 1e-12
    return base, coef


def solve(hl, nev: int, rk: int, ncycle: int, npow: int, nals: int, solvtol: float = 0.0, base=None, coef=None,
          bounds=None, resfile: str | None = None, seed: int = 0):
    """Run up to ncycle GPU power cycles on a block of nev vectors of rank rk.
    Returns (base, coef, eigv, bounds, history) with history the per-cycle
    relative rms eigenvalue change."""
    nbas = np.asarray(hl.nbas)
    if base is None:
        base, coef = product_guess(nbas, nev, rk, seed)
    if bounds is None:
        sb, sc = spectral_start(nbas, rk, seed)
        _, _, bounds = IT.spectral_range(sb, sc, nbas, rk, hl, 10, 5)
    eigv = IT.qhq_diag(base, coef, nbas, rk, nev, hl)
    history = []
    for i in range(ncycle):
        old = eigv.copy()
        esh = IT.block_shift(eigv, bounds[1])
        base, coef, eigv = IT.intertwine(base, coef, nbas, rk, nev, hl, eigv, npow, nals, True, 1, esh)
        delta = (old - eigv) / np.abs(eigv)
        rms = float(np.sqrt(np.sum(delta ** 2)) / nev)
        history.append(rms)
        if resfile is not None:
            from . import restart
            restart.save_psi(resfile, i + 1, bounds, eigv, delta, base, coef, nbas)
        if rms < solvtol:
            break
    return base, coef, eigv, bounds, history
