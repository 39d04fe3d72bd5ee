"""CPU oracle for the MLCP power-iteration hot path (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, and only as the checker.  The product
library under ``mlcp_gb300/`` never calls it.

The C code in ``mlcp_oracle.c`` restates the reference's CUDA algorithm
(src/intertwining.cu, src/als.cu, src/intertw_mvp.cu, src/intertw_lcv.cu)
in FP64.  The reference holds no golden vectors for this path, so the
restatement is pinned against the reference itself: ``ref_build.py``
compiles the reference's own FP64 CUDA library from its sources (where
they are staged) and ``Reference`` runs it in a child process, and the GPU
tests compare this oracle, the reference library and the GB300 library on
the same inputs (ALS: 1e-12; one power cycle: 1e-10).  Mathematical known
answers (dense diagonalisation, FP64 Lanczos fixtures under
``tests/golden/``) cover the host loops.

The Fortran host's own CPU routines are restated beside it: reduc_ALS
(``reduc_als``) and the CPU power solver, solver pals at lowmem 4
(``pals_pow3``, ``pals_ortho2``, ``pals_prodhv2``, ``pals_sumlcvec2``,
``pals_diagonalize``, ``pals_cycle``), which agree with the CUDA-algorithm
restatement stage by stage to rounding (``tests/test_oracle_pals.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libmlcp_oracle.so")
_lib: Optional[ctypes.CDLL] = None

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (FP contraction off: identical bits on x86 and Arm)."""
    src = os.path.join(_HERE, "mlcp_oracle.c")
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(src):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC", "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        L = _lib
        L.orc_alscpp.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_intertwine.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I, _D, _D,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, _D, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.orc_pow_als_block.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I, _D, _D,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.orc_gram_schmidt.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_gen_eig.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I, _D, _D,
                                  ctypes.c_int, ctypes.c_int, _D, _D, ctypes.c_int]
        L.orc_vector_updates.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, _D,
                                         ctypes.c_int, ctypes.c_int]
        L.orc_cp_dot.restype = ctypes.c_double
        L.orc_cp_dot.argtypes = [_D, _D, ctypes.c_int, _D, _D, ctypes.c_int, _I, ctypes.c_int]
        L.orc_als_batched.argtypes = [ctypes.c_int, ctypes.POINTER(_D), ctypes.POINTER(_D), _I, ctypes.c_int,
                                      _I, _I, ctypes.c_int, ctypes.c_int]
        L.orc_set_penalty_factor.argtypes = [ctypes.c_double]
        L.orc_set_cycle_penalties.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_set_rhs_fp32.argtypes = [ctypes.c_int]
        L.orc_sygv.restype = ctypes.c_int
        L.orc_sygv.argtypes = [ctypes.c_int, _D, _D, _D, _D]
        L.orc_rayleigh_quotient.restype = ctypes.c_double
        L.orc_rayleigh_quotient.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, _I, _I, _D, _D, ctypes.c_int]
        L.orc_update_opermat.argtypes = [ctypes.c_int, _D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int, _D, _D]
        L.orc_spectral_range.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I,
                                         _D, _D, ctypes.c_int, _D]
        L.orc_qhq_diag.argtypes = [_D, _D, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _I, _I, _D,
                                   _D, ctypes.c_int, _D, ctypes.c_int]
        L.orc_reduc_als.restype = ctypes.c_int
        L.orc_reduc_als.argtypes = [_D, _D, ctypes.c_int, _D, _D, ctypes.c_int, _I, ctypes.c_int, ctypes.c_int]
        L.orc_reduc_als_batched.restype = ctypes.c_int
        L.orc_reduc_als_batched.argtypes = [ctypes.c_int, ctypes.POINTER(_D), ctypes.POINTER(_D), _I,
                                            ctypes.POINTER(_D), ctypes.POINTER(_D), _I, _I, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_int]
        c_i, c_d = ctypes.c_int, ctypes.c_double
        for name in ("orc_pals_pow3", "orc_pals_ortho2", "orc_pals_ortho3", "orc_pals_prodhv2", "orc_pals_prodhv3",
                     "orc_pals_sumlcvec2", "orc_pals_sumlcvec3", "orc_pals_diagonalize", "orc_pals_cycle"):
            getattr(L, name).restype = c_i
        L.orc_pals_pow3.argtypes = [_D, _D, _I, c_i, c_i, _I, c_i, _I, _I, _D, _D, c_i, c_i, c_i, c_d, c_i]
        L.orc_pals_pow.restype = c_i
        L.orc_pals_pow.argtypes = [_D, _D, _I, c_i, c_i, _I, c_i, _I, _I, _D, _D, c_i, c_i, c_i, c_d, c_i, c_i]
        for name in ("orc_pals_ortho2", "orc_pals_ortho3"):
            getattr(L, name).argtypes = [_D, _D, _I, c_i, c_i, _I, c_i, c_i]
        for name in ("orc_pals_prodhv2", "orc_pals_prodhv3"):
            getattr(L, name).argtypes = [_D, _D, _D, _D, _I, c_i, c_i, _I, _I, _D, _D, c_i, c_i, c_d, c_i]
        for name in ("orc_pals_sumlcvec2", "orc_pals_sumlcvec3"):
            getattr(L, name).argtypes = [_D, _D, _I, c_i, c_i, _I, _D, c_i, c_i]
        L.orc_pals_diagonalize.argtypes = [_D, _D, _I, c_i, c_i, _I, _I, _I, _D, _D, c_i, c_i, c_i, _D, _D, c_i]
        L.orc_pals_cycle.argtypes = [_D, _D, _I, c_i, c_i, _I, c_i, _I, _I, _D, _D, c_i, c_i, c_i, c_i, c_i, c_i,
                                     c_d, _D, c_i]
        L.orc_prodhv.argtypes = [_D, _D, _I, c_i, c_i, _I, _I, _D, _D, c_i, c_i, c_d, _D, _D]
        L.orc_powr_recurse.restype = c_i
        L.orc_powr_recurse.argtypes = [_D, _D, _I, c_i, c_i, _I, _I, _D, _D, c_i, c_i, c_d, c_i]
        L.orc_gramortho.restype = c_i
        L.orc_gramortho.argtypes = [_D, _D, _I, c_i, c_i, _I, c_i, c_i, c_i]
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def _ip(a: np.ndarray):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_I)


def als(coef: np.ndarray, base: np.ndarray, nbas, rF: int, rG: int, nals: int):
    """Reference alscpp_ semantics.  ``base`` is (rF+rG, nD) row = term; returns
    the reduced (coef[rF], base[rF, nD]) as new arrays.  As in the reference,
    the target is processed in blocks of rF terms, so rG must be a multiple of
    rF (callers pad with zero-weight terms, src/GPUIterate.f90:249-268)."""
    if rG % rF != 0:
        raise ValueError(f"rG={rG} is not a multiple of rF={rF}; pad the target (see pad_target)")
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    lib().orc_alscpp(_dp(coef), _dp(base), _ip(nb), len(nb), rF, rG, nals)
    return coef[:rF].copy(), base[:rF].copy()


def reduc_als(gcoef, gbase, fcoef, fbase, nbas, nitn: int):
    """The Fortran host's CPU ALS reduction reduc_ALS (src/REDUCTIONML.f90:
    593-731): F fitted to G by nitn sweeps, penalty 1e-15 max c_G.  Returns
    the new (coef, base) of F; raises when a weight comes out NaN."""
    gc = np.ascontiguousarray(gcoef, dtype=np.float64)
    gb = np.ascontiguousarray(gbase, dtype=np.float64)
    fc = np.ascontiguousarray(fcoef, dtype=np.float64).copy()
    fb = np.ascontiguousarray(fbase, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    if lib().orc_reduc_als(_dp(gc), _dp(gb), gc.size, _dp(fc), _dp(fb), fc.size, _ip(nb), len(nb), nitn):
        raise FloatingPointError("reduc_ALS: NaN weight (the reference restarts from a random vector)")
    return fc, fb


def reduc_als_batched(gcoefs, gbases, fcoefs, fbases, nbas, nitn: int, nthreads: int = 0) -> int:
    """reduc_ALS on independent vectors, OpenMP over vectors; F in place.
    Returns the number of vectors that hit a NaN weight."""
    n = len(gcoefs)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    gcp = (_D * n)(*[_dp(c) for c in gcoefs])
    gbp = (_D * n)(*[_dp(b) for b in gbases])
    fcp = (_D * n)(*[_dp(c) for c in fcoefs])
    fbp = (_D * n)(*[_dp(b) for b in fbases])
    rg = np.ascontiguousarray([c.size for c in gcoefs], dtype=np.int32)
    rf = np.ascontiguousarray([c.size for c in fcoefs], dtype=np.int32)
    return int(lib().orc_reduc_als_batched(n, gcp, gbp, _ip(rg), fcp, fbp, _ip(rf), _ip(nb), len(nb), nitn,
                                           nthreads))


def pad_target(coef: np.ndarray, base: np.ndarray, rF: int, rG: int, seed: int = 0):
    """Pad the target to a multiple of rF with random-factor, zero-weight
    terms, as the reference's GPU_ALS_AB does (src/GPUIterate.f90:249-268)."""
    rGa = (rG + rF - 1) // rF * rF
    if rGa == rG:
        return coef.copy(), base.copy(), rG
    rng = np.random.default_rng(seed)
    extra = rGa - rG
    c = np.concatenate([coef[:rF + rG], np.zeros(extra)])
    b = np.vstack([base[:rF + rG], rng.uniform(0.0, 1.0, size=(extra, base.shape[1]))])
    return c, b, rGa


def als_batched(coefs, bases, nbas, rFs, rGs, nals: int, nthreads: int = 0):
    """Independent explicit-G reductions, OpenMP over vectors; in place."""
    n = len(coefs)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    cp = (_D * n)(*[_dp(c) for c in coefs])
    bp = (_D * n)(*[_dp(b) for b in bases])
    rf = np.ascontiguousarray(rFs, dtype=np.int32)
    rg = np.ascontiguousarray(rGs, dtype=np.int32)
    lib().orc_als_batched(n, cp, bp, _ip(nb), len(nb), _ip(rf), _ip(rg), nals, nthreads)


def intertwine(base, coef, nbas, rk, nbloc, hl, eigv, npow, nals, update=True, ishift=1, Eshift=0.0, ncpu=0):
    """Reference intertwinecpp_ semantics on copies; returns (base, coef, eigv)."""
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    eig = np.ascontiguousarray(eigv, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    lib().orc_intertwine(_dp(base), _dp(coef), _ip(nb), rk, len(nb), nbloc, _ip(hl.opid), _ip(hl.mptr),
                         _dp(hl.coef), _dp(hl.mat), hl.opid.size, hl.mptr.size, hl.mat.size, _dp(eig),
                         npow, ncpu, nals, int(bool(update)), ishift, float(Eshift))
    return base, coef, eig


def pow_als_block(base, coef, nbas, rk, nbloc, hl, npow, ishift=1, Eshift=0.0, nthreads=0):
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    lib().orc_pow_als_block(_dp(base), _dp(coef), _ip(nb), rk, len(nb), nbloc, _ip(hl.opid), _ip(hl.mptr),
                            _dp(hl.coef), _dp(hl.mat), hl.nterms, npow, ishift, float(Eshift), nthreads)
    return base, coef


def gram_schmidt(base, coef, nbas, rk, nbloc, nals):
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    lib().orc_gram_schmidt(_dp(base), _dp(coef), _ip(nb), rk, len(nb), nbloc, nals)
    return base, coef


def gen_eig(base, coef, nbas, rk, nbloc, hl, nals, nthreads=0):
    base = np.ascontiguousarray(base, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    eig = np.zeros(nbloc)
    U = np.zeros(nbloc * nbloc)
    lib().orc_gen_eig(_dp(base), _dp(coef), _ip(nb), rk, len(nb), nbloc, _ip(hl.opid), _ip(hl.mptr),
                      _dp(hl.coef), _dp(hl.mat), hl.nterms, nals, _dp(eig), _dp(U), nthreads)
    return eig, U.reshape(nbloc, nbloc).T.copy()  # U[:, i] = eigenvector i


def vector_updates(base, coef, nbas, rk, nbloc, U, nals, nthreads=0):
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    Ucm = np.ascontiguousarray(np.asarray(U, dtype=np.float64).T)  # column-major
    lib().orc_vector_updates(_dp(base), _dp(coef), _ip(nb), rk, len(nb), nbloc, _dp(Ucm), nals, nthreads)
    return base, coef


def rayleigh_quotient(base, coef, nbas, hl) -> float:
    """Reference RayleighQuotient2 (src/BlockUtils.f90:658-688): <v|H|v>/<v|v>."""
    base = np.ascontiguousarray(base, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    return lib().orc_rayleigh_quotient(_dp(base), _dp(coef), _ip(nb), coef.size, len(nb), _ip(hl.opid),
                                       _ip(hl.mptr), _dp(hl.coef), _dp(hl.mat), hl.nterms)


def qhq_diag(base, coef, nbas, rk, nbloc, hl, nconv=0, qhqd=None, nthreads=0):
    """Reference GetQHQdiag (src/BlockUtils.f90:385-408): Rayleigh quotients of
    vectors nconv..nbloc-1; qhqd (copied) keeps its entries below nconv."""
    base = np.ascontiguousarray(base, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    out = np.zeros(nbloc) if qhqd is None else np.ascontiguousarray(qhqd, dtype=np.float64).copy()
    lib().orc_qhq_diag(_dp(base), _dp(coef), _ip(nb), rk, len(nb), nbloc, nconv, _ip(hl.opid), _ip(hl.mptr),
                       _dp(hl.coef), _dp(hl.mat), hl.nterms, _dp(out), nthreads)
    return out


def update_opermat(imode, base, coef, nbas, rk, nbloc, xmats):
    """Reference UpdateOperMat (src/Updater.f90:110-151) for the operators
    xmats (each packed upper-triangular, n(n+1)/2) of mode imode (1-based);
    returns the packed nbloc x nbloc matrices, one row per operator."""
    base = np.ascontiguousarray(base, dtype=np.float64)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    xm = np.ascontiguousarray(np.atleast_2d(xmats), dtype=np.float64)
    out = np.zeros((xm.shape[0], nbloc * (nbloc + 1) // 2))
    lib().orc_update_opermat(imode, _dp(base), _dp(coef), _ip(nb), rk, len(nb), nbloc, xm.shape[0], _dp(xm),
                             _dp(out))
    return out


def unpack_sym(v, n):
    """Symmetric matrix from its packed upper triangle (column by column)."""
    M = np.zeros((n, n))
    k = 0
    for j in range(n):
        for i in range(j + 1):
            M[i, j] = M[j, i] = v[k]
            k += 1
    return M


def spectral_start(nbas, rk, seed=0):
    """The two starting vectors of GetSpectralRange (src/Solver.f90:583-606):
    the first (lower guess) and last (upper guess) basis function of every
    mode, 1e-15 elsewhere, weight 1, plus (more than two modes, rk > 1) the
    same rk - 1 seeded random terms (uniform -0.5..0.5, normalised per mode)
    with weight 1e-7.  Returns (base, coef) of the 2 x rk terms."""
    nbas = np.asarray(nbas, dtype=np.int32)
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


def spectral_range(base, coef, nbas, rk, hl, npow, ncyc):
    """Reference GetSpectralRange (more than two modes) from the starting
    vectors; returns (base, coef, bounds) with the padded bounds."""
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    bounds = np.zeros(2)
    lib().orc_spectral_range(_dp(base), _dp(coef), _ip(nb), rk, len(nb), npow, ncyc, _ip(hl.opid), _ip(hl.mptr),
                             _dp(hl.coef), _dp(hl.mat), hl.nterms, _dp(bounds))
    return base, coef, bounds


def cp_dense(base, coef, nbas):
    """The full tensor of a CP vector, flattened (mode 0 slowest)."""
    nbas = [int(n) for n in nbas]
    offs = np.concatenate([[0], np.cumsum(nbas)])
    base = np.asarray(base, dtype=np.float64).reshape(-1, offs[-1])
    coef = np.asarray(coef, dtype=np.float64).ravel()
    out = np.zeros(int(np.prod(nbas)))
    for r in range(coef.size):
        t = np.array([coef[r]])
        for d in range(len(nbas)):
            t = np.multiply.outer(t, base[r, offs[d]:offs[d + 1]]).ravel()
        out += t
    return out


def diagonalize_dense(base, coef, nbas, rk, nbloc, hl, nals=0):
    """Reference Diagonalize with intw = .FALSE. (src/BlockUtils.f90:184-225)
    on small cases through dense tensors: A = <Q_j|H|Q_i> and S = <Q_j|Q_i>
    (GetQHQ, GetOverlaps, H exact), the generalised eigenproblem
    (SolveGenEigval: ascending; each eigenvector scaled to X^T S X = I and its
    largest-magnitude entry made positive, the library's convention), then
    UpdateVecs (:437-475): for two modes the SVD reduction of
    sum_i U(i, m) Q_i to at most rk terms and NORMCOEF; for more modes the
    ALS update of the restated vector updates from the old vectors (nals
    sweeps).  Returns (base, coef, eigv, U); for two modes base/coef list the
    new vectors' (base, coef) pairs."""
    import scipy.linalg
    from mlcp_gb300 import hoplist as H
    nD = int(np.sum(nbas))
    base = np.asarray(base, dtype=np.float64).reshape(nbloc * rk, nD)
    coef = np.asarray(coef, dtype=np.float64).ravel()
    Qd = np.array([cp_dense(base[i * rk:(i + 1) * rk], coef[i * rk:(i + 1) * rk], nbas) for i in range(nbloc)])
    Hd = H.dense_hamiltonian(hl)
    A = Qd @ Hd @ Qd.T
    S = Qd @ Qd.T
    lam, U = scipy.linalg.eigh(0.5 * (A + A.T), 0.5 * (S + S.T))
    for m in range(nbloc):
        if U[np.argmax(np.abs(U[:, m])), m] < 0:
            U[:, m] = -U[:, m]
    if len(nbas) == 2:
        vecs = []
        for m in range(nbloc):
            w = (U[:, m][:, None] * coef.reshape(nbloc, rk)).ravel()
            b, c = reduc_svd(base, w, nbas, rk)
            vecs.append(normcoef(b, c, nbas))
        return vecs, None, lam, U
    if nals > 0:
        nb, nc = vector_updates(base, coef, nbas, rk, nbloc, U, nals)
        return nb, nc, lam, U
    return base.copy(), coef.copy(), lam, U


def cp2d_dense(base, coef, nbas):
    """Reference CP2DtoMat (src/SepdRepn.f90:518-558): the nr x nc matrix
    sum_k c_k a_k b_k^T of a two-mode CP vector."""
    nr, nc = int(nbas[0]), int(nbas[1])
    base = np.asarray(base, dtype=np.float64).reshape(-1, nr + nc)
    coef = np.asarray(coef, dtype=np.float64).ravel()
    return (base[:, :nr] * coef[:, None]).T @ base[:, nr:]


def reduc_svd(base, coef, nbas, rF, redtol=1.0e-12):
    """Reference reduc_SVDa (src/REDUCTIONML.f90:296-333): CP2DtoMat, the SVD
    (SolveWithSVD, src/LinAlg.f90:432-466, LAPACK through numpy), ncomp = the
    leading singular values >= redtol * s_1 (at least one), nrk =
    min(nr, nc, rF, ncomp) and RebuildfromSVD (src/REDUCTIONML.f90:394-439):
    coef = s_i, mode 1 = U(:, i), mode 2 = V(:, i).  Returns (base, coef)
    with nrk terms."""
    nr, nc = int(nbas[0]), int(nbas[1])
    U, s, Vt = np.linalg.svd(cp2d_dense(base, coef, nbas), full_matrices=False)
    cut = redtol * s[0]
    ncomp = 1
    for i in range(1, s.size):
        if abs(s[i]) < cut:
            break
        ncomp = i + 1
    nrk = min(nr, nc, rF, ncomp)
    return np.concatenate([U[:, :nrk].T, Vt[:nrk, :]], axis=1), s[:nrk].copy()


def normcoef(base, coef, nbas):
    """Reference NORMCOEF (src/MODVECVECML.f90:295-352): unit factors with
    their norms moved into the weights, then the weights divided by the
    vector's norm.  Returns copies."""
    nbas = np.asarray(nbas)
    offs = np.concatenate([[0], np.cumsum(nbas)])
    base = np.array(base, dtype=np.float64).reshape(-1, int(nbas.sum()))
    coef = np.array(coef, dtype=np.float64).ravel()
    G = np.ones((coef.size, coef.size))
    for d in range(nbas.size):
        blk = base[:, offs[d]:offs[d + 1]]
        nrm = np.linalg.norm(blk, axis=1)
        blk /= nrm[:, None]
        coef *= nrm
        G *= blk @ blk.T
    return base, coef / np.sqrt(abs(coef @ G @ coef))


def prodhv_2mode(base, coef, nbas, hl, eshift):
    """Reference PRODHV (src/MODHVECML.f90:50-111) with ishift = 1: the terms
    of H v followed by those of -eshift v, for a two-mode v."""
    nr = int(nbas[0])
    base = np.asarray(base, dtype=np.float64).reshape(-1, int(np.sum(nbas)))
    coef = np.asarray(coef, dtype=np.float64).ravel()
    bs, cs = [], []
    for t in range(hl.nterms):
        h1, h2 = hl.operator(t, 0), hl.operator(t, 1)
        bs.append(np.concatenate([base[:, :nr] @ h1.T, base[:, nr:] @ h2.T], axis=1))
        cs.append(hl.coef[t] * coef)
    bs.append(base.copy())
    cs.append(-eshift * coef)
    return np.concatenate(bs), np.concatenate(cs)


def spectral_range_2mode(nbas, rk, hl, npow, ncyc):
    """Reference GetSpectralRange (src/Solver.f90:563-654), two-mode branch:
    rank-1 starting vectors, PowrRecurse (src/BlockPower.f90:49-73: PRODHV,
    reduc by SVD to at most rk terms with redtol 1e-12, NORMCOEF) and the
    Rayleigh quotients.  Returns ([(base, coef)] * 2, padded bounds)."""
    b0, c0 = spectral_start(nbas, rk)
    vecs = [(b0[j * rk:j * rk + 1].copy(), c0[j * rk:j * rk + 1].copy()) for j in range(2)]
    bounds = np.array([rayleigh_quotient(b, c, nbas, hl) for b, c in vecs])
    shift = [0.5 * (bounds[0] + bounds[1]), 0.0]
    for _ in range(ncyc):
        for j in range(2):
            b, c = vecs[j]
            for _ in range(npow):
                wb, wc = prodhv_2mode(b, c, nbas, hl, shift[j])
                b, c = reduc_svd(wb, wc, nbas, rk)
                b, c = normcoef(b, c, nbas)
            vecs[j] = (b, c)
            bounds[j] = rayleigh_quotient(b, c, nbas, hl)
        shift[0] = 0.5 * (bounds[0] + bounds[1])
    pad = 0.001 * (bounds[1] - bounds[0])
    return vecs, np.array([bounds[0] - pad, bounds[1] + pad])


def sort_vecs(base, coef, rk, eigv, nconv, eref):
    """Reference SortVecs (src/BlockUtils.f90:520-583) on copies: vectors in
    increasing |eigv - Eref| (ties keep their order), eigv permuted alike, and
    nconv cut back to the first converged vector that moved.  Returns
    (base, coef, eigv, nconv)."""
    eigv = np.asarray(eigv, dtype=np.float64)
    nbloc = eigv.size
    ix = np.argsort(np.abs(eigv - eref), kind="stable")
    base = np.asarray(base, dtype=np.float64).reshape(nbloc, rk, -1)[ix].reshape(nbloc * rk, -1).copy()
    coef = np.asarray(coef, dtype=np.float64).reshape(nbloc, rk)[ix].reshape(-1).copy()
    moved = [i for i in range(nconv) if ix[i] != i]
    return base, coef, eigv[ix].copy(), (moved[0] if moved else nconv)


def fortran_records(path):
    """The records of a gfortran unformatted sequential file, as bytes: each
    record is a 4-byte little-endian length, the data, and the length again.
    Raises ValueError on a broken frame."""
    import struct
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        if pos + 4 > len(data):
            raise ValueError("truncated record marker")
        (n,) = struct.unpack_from("<i", data, pos)
        if n < 0 or pos + 8 + n > len(data):
            raise ValueError("bad record length")
        (m,) = struct.unpack_from("<i", data, pos + 4 + n)
        if m != n:
            raise ValueError("record markers differ")
        out.append(data[pos + 4:pos + 4 + n])
        pos += 8 + n
    return out


def psi_write(path, isavi, bounds, eigv, delta, nbas, ranks, coef, base) -> None:
    """Reference SavePsiFile (src/Restart.f90:759-793) restated: the WRITE
    statements (isavi, nev), bounds, eigv, delta and per vector
    (ndof, nrk), nbas, coef, base, as gfortran frames them.  coef/base hold
    the vectors back to back (base: nD values per term)."""
    import struct
    nb = np.asarray(nbas, dtype="<i4")
    nD = int(nb.sum())
    eigv = np.asarray(eigv, dtype="<f8")
    coef = np.asarray(coef, dtype="<f8").ravel()
    base = np.asarray(base, dtype="<f8").ravel()
    recs = [struct.pack("<ii", int(isavi), eigv.size), np.asarray(bounds, dtype="<f8").tobytes(), eigv.tobytes(),
            np.asarray(delta, dtype="<f8").tobytes()]
    t = 0
    for r in ranks:
        r = int(r)
        recs += [struct.pack("<ii", nb.size, r), nb.tobytes(), coef[t:t + r].tobytes(),
                 base[t * nD:(t + r) * nD].tobytes()]
        t += r
    with open(path, "wb") as f:
        for rec in recs:
            f.write(struct.pack("<i", len(rec)) + rec + struct.pack("<i", len(rec)))


def psi_read(path):
    """Reference ReadPsiFile (src/Restart.f90:614-731) restated without its
    checks against the caller's block: returns a dict with isavi, bounds,
    eigv, delta, nbas (per vector), ranks, coef and base, read as a Fortran
    READ reads (a record longer than the list is accepted)."""
    import struct
    recs = fortran_records(path)
    isavi, nev = struct.unpack_from("<ii", recs[0])
    out = {"isavi": isavi, "bounds": np.frombuffer(recs[1], "<f8", 2).copy(),
           "eigv": np.frombuffer(recs[2], "<f8", nev).copy(), "delta": np.frombuffer(recs[3], "<f8", nev).copy(),
           "nbas": [], "ranks": [], "coef": [], "base": []}
    k = 4
    for _ in range(nev):
        ndof, nrk = struct.unpack_from("<ii", recs[k])
        nb = np.frombuffer(recs[k + 1], "<i4", ndof).copy()
        out["nbas"].append(nb)
        out["ranks"].append(nrk)
        out["coef"].append(np.frombuffer(recs[k + 2], "<f8", nrk))
        out["base"].append(np.frombuffer(recs[k + 3], "<f8", nrk * int(nb.sum())))
        k += 4
    out["coef"] = np.concatenate(out["coef"]) if nev else np.zeros(0)
    out["base"] = np.concatenate(out["base"]) if nev else np.zeros(0)
    out["ranks"] = np.asarray(out["ranks"], dtype=np.int32)
    return out


def cp_dot(vb, vc, wb, wc, nbas) -> float:
    vb = np.ascontiguousarray(vb, dtype=np.float64)
    vc = np.ascontiguousarray(vc, dtype=np.float64)
    wb = np.ascontiguousarray(wb, dtype=np.float64)
    wc = np.ascontiguousarray(wc, dtype=np.float64)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    return lib().orc_cp_dot(_dp(vb), _dp(vc), vc.size, _dp(wb), _dp(wc), wc.size, _ip(nb), len(nb))


# Penalty factors of the reference's two builds (src/als.cu:248-267).
PEN_FP64 = 1.0e-10
PEN_FP32 = 1.0e-5


def set_cycle_penalties(mvp: float = PEN_FP64, gs: float = PEN_FP64, upd: float = PEN_FP64) -> None:
    """Penalty factors of the cycle's stages (power sweeps and H-applications,
    Gram-Schmidt, vector updates).  Defaults restore the FP64 rule."""
    lib().orc_set_cycle_penalties(mvp, gs, upd)


def set_penalty_factor(f: float) -> None:
    lib().orc_set_penalty_factor(f)


def set_rhs_fp32(on: bool) -> None:
    """Round every ALS right-hand side to FP32 before its solve (test knob:
    the drift of an FP64 trajectory under FP32-level noise in b)."""
    lib().orc_set_rhs_fp32(1 if on else 0)


def sygv(A: np.ndarray, B: np.ndarray):
    """A x = w B x; returns (w ascending, X with columns = eigenvectors)."""
    n = A.shape[0]
    Acm = np.ascontiguousarray(np.asarray(A, dtype=np.float64).T)
    Bcm = np.ascontiguousarray(np.asarray(B, dtype=np.float64).T)
    w = np.zeros(n)
    X = np.zeros(n * n)
    info = lib().orc_sygv(n, _dp(Acm), _dp(Bcm), _dp(w), _dp(X))
    return w, X.reshape(n, n).T.copy(), info


# --- the Fortran host's CPU solver (solver pals, src/Solver.f90:508-538, lowmem 4) ---
# A block is the terms of vector 0, then vector 1, ...; ``ranks`` gives each
# vector's number of terms (default: rk for all).  Every routine works on
# copies and raises on a NaN weight, where the reference aborts.

def _block(base, coef, nbloc, rk, ranks):
    base = np.ascontiguousarray(base, dtype=np.float64).copy()
    coef = np.ascontiguousarray(coef, dtype=np.float64).copy()
    rv = np.full(nbloc, rk, dtype=np.int32) if ranks is None else np.ascontiguousarray(ranks, dtype=np.int32)
    if rv.size != nbloc or int(rv.sum()) != coef.size:
        raise ValueError(f"ranks {rv.tolist()} do not cover {coef.size} terms")
    return base, coef, rv


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise FloatingPointError(f"{what}: {'eigensolve failed' if rc < 0 else 'NaN weight'}")


def pals_pow(base, coef, nbas, rk, nbloc, hl, npow, ishift=1, Eshift=0.0, nconv=0, ranks=None, nthreads=0,
             lowmem=4):
    """ALS_POW_alg (src/ALSPow.f90:83-112) on vectors nconv..nbloc-1: lowmem 0
    ALS_POW0, 1 ALS_POW1, 2 ALS_POW2, 3 and 4 ALS_POW3."""
    if lowmem not in (0, 1, 2, 3, 4):
        raise ValueError("lowmem must be 0-4")
    base, coef, rv = _block(base, coef, nbloc, rk, ranks)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    _check(lib().orc_pals_pow(_dp(base), _dp(coef), _ip(nb), len(nb), nbloc, _ip(rv), nconv, _ip(hl.opid),
                              _ip(hl.mptr), _dp(hl.coef), _dp(hl.mat), hl.nterms, npow, ishift, float(Eshift), lowmem,
                              nthreads), f"ALS_POW (lowmem {lowmem})")
    return base, coef


def pals_pow3(base, coef, nbas, rk, nbloc, hl, npow, ishift=1, Eshift=0.0, nconv=0, ranks=None, nthreads=0):
    """ALS_POW3 (src/ALSPow.f90:569-660) on vectors nconv..nbloc-1."""
    base, coef, rv = _block(base, coef, nbloc, rk, ranks)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    _check(lib().orc_pals_pow3(_dp(base), _dp(coef), _ip(nb), len(nb), nbloc, _ip(rv), nconv, _ip(hl.opid),
                               _ip(hl.mptr), _dp(hl.coef), _dp(hl.mat), hl.nterms, npow, ishift, float(Eshift),
                               nthreads), "ALS_POW3")
    return base, coef


def pals_ortho2(base, coef, nbas, rk, nbloc, nitn, ranks=None, nthreads=0, lowmem=4):
    """ALS_ORTHO_2 (src/ALSUtils.f90:156-377); ALS_ORTHO_3 (:381-528) with lowmem 3."""
    base, coef, rv = _block(base, coef, nbloc, rk, ranks)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    fn = lib().orc_pals_ortho3 if lowmem == 3 else lib().orc_pals_ortho2
    _check(fn(_dp(base), _dp(coef), _ip(nb), len(nb), nbloc, _ip(rv), nitn, nthreads),
           "ALS_ORTHO_3" if lowmem == 3 else "ALS_ORTHO_2")
    return base, coef


def pals_prodhv2(base, coef, nbas, hl, nitn, ishift=0, Eshift=0.0, lowmem=4):
    """PRODHV_ALS2 (src/ALSPow.f90:664-780): ALS fit of (H - Eshift) F, F's
    rank; PRODHV_ALS3 (:784-865) with lowmem 3."""
    fb = np.ascontiguousarray(base, dtype=np.float64)
    fc = np.ascontiguousarray(coef, dtype=np.float64)
    ob, oc = np.zeros_like(fb), np.zeros_like(fc)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    fn = lib().orc_pals_prodhv3 if lowmem == 3 else lib().orc_pals_prodhv2
    _check(fn(_dp(fb), _dp(fc), _dp(ob), _dp(oc), _ip(nb), len(nb), fc.size, _ip(hl.opid), _ip(hl.mptr),
              _dp(hl.coef), _dp(hl.mat), hl.nterms, ishift, float(Eshift), nitn),
           "PRODHV_ALS3" if lowmem == 3 else "PRODHV_ALS2")
    return ob, oc


def pals_sumlcvec2(base, coef, nbas, rk, nbloc, U, nitn, ranks=None, nthreads=0, lowmem=4):
    """UpdateVecs2 with ALS_SUMLCVEC_2 (ALS_SUMLCVEC_3 with lowmem 3):
    vector i <- fit of sum_l U[l, i] Q_l."""
    base, coef, rv = _block(base, coef, nbloc, rk, ranks)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    Ucm = np.ascontiguousarray(np.asarray(U, dtype=np.float64).T)
    fn = lib().orc_pals_sumlcvec3 if lowmem == 3 else lib().orc_pals_sumlcvec2
    _check(fn(_dp(base), _dp(coef), _ip(nb), len(nb), nbloc, _ip(rv), _dp(Ucm), nitn, nthreads),
           "ALS_SUMLCVEC_3" if lowmem == 3 else "ALS_SUMLCVEC_2")
    return base, coef


def pals_diagonalize(base, coef, nbas, rk, nbloc, hl, nitn, ranks=None, nthreads=0, lowmem=4):
    """Diagonalize with intertwining (src/BlockUtils.f90:184-225); returns
    (base, coef, eigenvalues, U with U[:, i] = eigenvector i)."""
    if nitn < 1:
        raise ValueError("Diagonalize with intertwining needs nitn >= 1 (PRODHV_ALS2 returns no H Q_i otherwise)")
    base, coef, rv = _block(base, coef, nbloc, rk, ranks)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    eig = np.zeros(nbloc)
    U = np.zeros(nbloc * nbloc)
    _check(lib().orc_pals_diagonalize(_dp(base), _dp(coef), _ip(nb), len(nb), nbloc, _ip(rv), _ip(hl.opid),
                                      _ip(hl.mptr), _dp(hl.coef), _dp(hl.mat), hl.nterms, nitn, lowmem, _dp(eig),
                                      _dp(U), nthreads), "Diagonalize")
    return base, coef, eig, U.reshape(nbloc, nbloc).T.copy()


def pals_cycle(base, coef, nbas, rk, nbloc, hl, eigv, npow, nals, update=True, ishift=1, Eshift=0.0, nconv=0,
               ranks=None, nthreads=0, lowmem=4):
    """One cycle of the Fortran host's CPU solver: ALS_POW_alg, ALS_ORTHO_alg
    and the diagonalisation at lowmem 0-4 (the _3 forms at lowmem 3, the _2
    forms otherwise); returns (base, coef, eigv)."""
    if lowmem not in (0, 1, 2, 3, 4):
        raise ValueError("lowmem must be 0-4")
    if update and nals < 1:
        raise ValueError("the cycle's diagonalisation needs nals >= 1 (PRODHV_ALS2 returns no H Q_i otherwise)")
    base, coef, rv = _block(base, coef, nbloc, rk, ranks)
    eig = np.ascontiguousarray(eigv, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    _check(lib().orc_pals_cycle(_dp(base), _dp(coef), _ip(nb), len(nb), nbloc, _ip(rv), nconv, _ip(hl.opid),
                                _ip(hl.mptr), _dp(hl.coef), _dp(hl.mat), hl.nterms, npow, nals, lowmem,
                                int(bool(update)), ishift, float(Eshift), _dp(eig), nthreads), "pals cycle")
    return base, coef, eig


# --- the Fortran host's plain power solver (solver powr), reduc = reduc_ALS ---

def prodhv(base, coef, nbas, hl, ishift=0, Eshift=0.0):
    """PRODHV (src/MODHVECML.f90:50-110): the explicit (H - Eshift) F."""
    fb = np.ascontiguousarray(base, dtype=np.float64)
    fc = np.ascontiguousarray(coef, dtype=np.float64)
    rG = fc.size * (hl.nterms + (1 if ishift else 0))
    gb = np.zeros((rG, fb.shape[-1]))
    gc = np.zeros(rG)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    lib().orc_prodhv(_dp(fb), _dp(fc), _ip(nb), len(nb), fc.size, _ip(hl.opid), _ip(hl.mptr), _dp(hl.coef),
                     _dp(hl.mat), hl.nterms, ishift, float(Eshift), _dp(gb), _dp(gc))
    return gb, gc


def powr_recurse(base, coef, nbas, hl, npow, Eshift, nloop):
    """PowrRecurse (src/BlockPower.f90:49-73) on one vector (copies)."""
    fb = np.ascontiguousarray(base, dtype=np.float64).copy()
    fc = np.ascontiguousarray(coef, dtype=np.float64).copy()
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    _check(lib().orc_powr_recurse(_dp(fb), _dp(fc), _ip(nb), len(nb), fc.size, _ip(hl.opid), _ip(hl.mptr),
                                  _dp(hl.coef), _dp(hl.mat), hl.nterms, npow, float(Eshift), nloop), "PowrRecurse")
    return fb, fc


def gramortho(base, coef, nbas, rk, nbloc, nloop, k=0, ranks=None, nthreads=0):
    """GRAMORTHO (k = 0) / pGRAMORTHO (src/BlockUtils.f90:22-123)."""
    base, coef, rv = _block(base, coef, nbloc, rk, ranks)
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    _check(lib().orc_gramortho(_dp(base), _dp(coef), _ip(nb), len(nb), nbloc, _ip(rv), k, nloop, nthreads),
           "GRAMORTHO")
    return base, coef


# --- the reference's own FP64 CUDA library (oracle/ref_build.py, oracle/ref_run.py) ---

def reference_staged() -> bool:
    """True when the reference's CUDA sources are staged under oracle/_ref/src."""
    from . import ref_build
    return ref_build.staged()


def reference_built() -> bool:
    from . import ref_build
    return os.path.exists(ref_build.LIB)


class Reference:
    """The reference's FP64 CUDA entry points, served by a child process
    (``oracle/ref_run.py``; the reference resets the device after each call).

    ``als`` runs ``alscpp_`` (src/intertwining.cu:180) once per vector;
    ``intertwine`` runs one ``intertwinecpp_`` cycle (src/intertwining.cu:98).
    Both return the reference's outputs and the host wall time of each call.
    Test and baseline infrastructure only."""

    def __init__(self, timeout: float = 1800.0):
        import subprocess as sp
        import sys
        from . import ref_build
        if not os.path.exists(ref_build.LIB):
            raise RuntimeError("reference library not built (oracle/ref_build.py)")
        self.timeout = timeout
        env = dict(os.environ, OMP_NUM_THREADS="1")
        self.proc = sp.Popen([sys.executable, os.path.join(_HERE, "ref_run.py")], stdin=sp.PIPE, stdout=sp.PIPE,
                             env=env)

    def _call(self, req: dict) -> dict:
        import io
        import select
        import struct
        import time as _t
        buf = io.BytesIO()
        np.savez(buf, **req)
        data = buf.getvalue()
        self.proc.stdin.write(struct.pack("<Q", len(data)) + data)
        self.proc.stdin.flush()
        fd = self.proc.stdout.fileno()
        deadline = _t.monotonic() + self.timeout

        def read(n):
            out = bytearray()
            while len(out) < n:
                left = deadline - _t.monotonic()
                if left <= 0 or not select.select([fd], [], [], left)[0]:
                    self.close(kill=True)
                    raise TimeoutError("reference runner did not answer in time")
                chunk = os.read(fd, n - len(out))
                if not chunk:
                    raise RuntimeError(f"reference runner exited (code {self.proc.poll()})")
                out += chunk
            return bytes(out)
        (n,) = struct.unpack("<Q", read(8))
        rep = dict(np.load(io.BytesIO(read(n)), allow_pickle=False))
        if "error" in rep:
            raise RuntimeError(f"reference runner: {rep['error']}")
        return rep

    def als(self, coefs, bases, nbas, rF: int, rG: int, nals: int):
        """coefs (nv, rF+rG), bases (nv, rF+rG, nD): F then G per vector, as
        the host passes them to alscpp_.  Returns (coef (nv, rF), base (nv, rF,
        nD), seconds (nv))."""
        rep = self._call({"op": np.array("als"), "coef": np.asarray(coefs, dtype=np.float64),
                          "base": np.asarray(bases, dtype=np.float64),
                          "nbas": np.asarray(nbas, dtype=np.int32), "rF": np.array(rF), "rG": np.array(rG),
                          "nals": np.array(nals)})
        return rep["coef"], rep["base"], rep["seconds"]

    def intertwine(self, base, coef, nbas, rk, nbloc, hl, eigv, npow, nals, update=True, ishift=1, Eshift=0.0):
        """One intertwinecpp_ cycle; returns (base, coef, eigv, seconds)."""
        rep = self._call({"op": np.array("cycle"), "base": np.asarray(base, dtype=np.float64),
                          "coef": np.asarray(coef, dtype=np.float64), "eigv": np.asarray(eigv, dtype=np.float64),
                          "nbas": np.asarray(nbas, dtype=np.int32), "opid": np.asarray(hl.opid, dtype=np.int32),
                          "mptr": np.asarray(hl.mptr, dtype=np.int32),
                          "hcoef": np.asarray(hl.coef, dtype=np.float64),
                          "mat": np.asarray(hl.mat, dtype=np.float64), "rk": np.array(rk),
                          "nbloc": np.array(nbloc), "npow": np.array(npow), "nals": np.array(nals),
                          "update": np.array(bool(update)), "ishift": np.array(ishift),
                          "eshift": np.array(float(Eshift))})
        return rep["base"], rep["coef"], rep["eigv"], float(rep["seconds"])

    def close(self, kill: bool = False):
        if self.proc is None:
            return
        try:
            if kill:
                self.proc.kill()
            else:
                self.proc.stdin.close()
            self.proc.wait(timeout=60)
        except Exception:
            self.proc.kill()
        self.proc = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
