"""Hamiltonian operator lists (the ``HopList`` of the reference).

Reference layout (src/hoplist.h:2-7, src/ModeH.f90:909-1068): for T terms
over D modes, ``opid[t*D + d]`` (1-based) selects operator matrix
``mptr[opid-1]`` (1-based) inside ``mat``.  Every operator is an n x n
symmetric matrix in packed upper-triangular storage, element (r, c), r <= c,
at ``mat[mptr-1 + r + c*(c+1)/2]``.  ``coef[t]`` multiplies term t and is
applied on mode 0.  ``mptr`` lists, in order: the identity of each mode,
one diagonal ("eigen") operator per mode, compound operators, then the
unique primitive operators of each mode (src/ModeH.f90:974-1060).

This module builds such lists from operator tables in a harmonic-oscillator
basis (matrix elements from the ladder-operator algebra, equivalent to
src/OpFuncs.f90:193-267) and generates the seeded synthetic Hamiltonians the
benchmarks use.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np


@dataclass
class HopList:
    nbas: np.ndarray   # int32 [D], basis size per mode
    opid: np.ndarray   # int32 [T*D], 1-based operator index per (term, mode)
    mptr: np.ndarray   # int32 [nops], 1-based start of each operator in mat
    coef: np.ndarray   # float64 [T]
    mat: np.ndarray    # float64 [msize], packed upper-triangular operators

    @property
    def ndof(self) -> int:
        return int(self.nbas.size)

    @property
    def nterms(self) -> int:
        return int(self.coef.size)

    def operator(self, t: int, d: int) -> np.ndarray:
        """Dense n x n matrix of term t, mode d (for checks)."""
        n = int(self.nbas[d])
        s = int(self.mptr[self.opid[t * self.ndof + d] - 1]) - 1
        return unpack(self.mat[s:s + n * (n + 1) // 2], n)


def pack(M: np.ndarray) -> np.ndarray:
    """Packed upper-triangular, column-major: (r, c), r <= c, at r + c(c+1)/2."""
    n = M.shape[0]
    out = np.empty(n * (n + 1) // 2)
    for c in range(n):
        out[c * (c + 1) // 2:c * (c + 1) // 2 + c + 1] = M[:c + 1, c]
    return out


def unpack(v: np.ndarray, n: int) -> np.ndarray:
    M = np.zeros((n, n))
    for c in range(n):
        M[:c + 1, c] = v[c * (c + 1) // 2:c * (c + 1) // 2 + c + 1]
    return np.triu(M) + np.triu(M, 1).T


# ---------------------------------------------------------------------------
# Harmonic-oscillator operator matrices (dimensionless normal coordinates)
# ---------------------------------------------------------------------------

def ho_q_power(n: int, p: int) -> np.ndarray:
    """<i|q^p|j> in the n-function HO basis: q = (a + a^dagger)/sqrt(2).
    Computed in an (n+p)-function basis and truncated, which is exact because
    q^p only couples |i> to |i +- p>."""
    m = n + p + 1
    q = np.zeros((m, m))
    for i in range(m - 1):
        q[i, i + 1] = q[i + 1, i] = np.sqrt((i + 1) / 2.0)
    out = np.eye(m)
    for _ in range(p):
        out = out @ q
    return out[:n, :n].copy()


def ho_p2(n: int) -> np.ndarray:
    """<i|p^2|j>: q^2 with the sign of the |i -+ 2> couplings flipped."""
    m = ho_q_power(n, 2)
    for i in range(n - 2):
        m[i, i + 2] = -m[i, i + 2]
        m[i + 2, i] = -m[i + 2, i]
    return m


# ---------------------------------------------------------------------------
# HopList assembly
# ---------------------------------------------------------------------------

Term = Tuple[float, Dict[int, np.ndarray]]


def build_hoplist(nbas: Sequence[int], terms: List[Term], eigen_ops: Optional[List[np.ndarray]] = None) -> HopList:
    """Assemble a HopList from ``terms`` = [(coef, {mode: dense n x n operator})].
    Modes absent from a term get the identity.  Operators equal (bitwise) to a
    mode's diagonal eigen operator are referenced through the eigen slots;
    the other distinct operators of each mode become primitive slots."""
    nbas = np.asarray(nbas, dtype=np.int32)
    D = nbas.size
    if eigen_ops is None:
        eigen_ops = [np.zeros((int(n), int(n))) for n in nbas]
    mats: List[np.ndarray] = []
    for d in range(D):
        mats.append(pack(np.eye(int(nbas[d]))))
    for d in range(D):
        mats.append(pack(np.diag(np.diag(eigen_ops[d]))))
    prim: List[List[np.ndarray]] = [[] for _ in range(D)]
    opidx = np.zeros((len(terms), D), dtype=np.int64)  # 0 = identity, -1 = eigen, k>0 primitive k of mode
    for t, (_, ops) in enumerate(terms):
        for d, M in ops.items():
            pk = pack(np.asarray(M, dtype=np.float64))
            if np.array_equal(pk, mats[D + d]) and np.any(pk != 0):
                opidx[t, d] = -1
                continue
            for k, other in enumerate(prim[d]):
                if np.array_equal(other, pk):
                    opidx[t, d] = k + 1
                    break
            else:
                prim[d].append(pk)
                opidx[t, d] = len(prim[d])
    psum = np.concatenate([[0], np.cumsum([len(p) for p in prim])]).astype(np.int64)
    opid = np.zeros(len(terms) * D, dtype=np.int32)
    for t in range(len(terms)):
        for d in range(D):
            k = opidx[t, d]
            if k == 0:
                opid[t * D + d] = d + 1
            elif k < 0:
                opid[t * D + d] = D + d + 1
            else:
                opid[t * D + d] = 2 * D + psum[d] + k
    for d in range(D):
        mats.extend(prim[d])
    mptr = np.zeros(len(mats), dtype=np.int32)
    pos = 1
    for i, m in enumerate(mats):
        mptr[i] = pos
        pos += m.size
    mat = np.concatenate(mats).astype(np.float64)
    coef = np.array([c for c, _ in terms], dtype=np.float64)
    return HopList(nbas=nbas, opid=opid, mptr=mptr, coef=coef, mat=mat)


def _to_eigenbasis(nbas, single: List[np.ndarray], terms: List[Term]):
    """First-layer step (src/HamilSetup.f90:570-645): diagonalise each mode's
    one-mode operator and transform every operator of that mode.  Term t < D
    must be mode t's one-mode term; it becomes the diagonal eigen operator."""
    vecs = []
    eig_ops = []
    for d, h in enumerate(single):
        w, V = np.linalg.eigh(h)
        for j in range(V.shape[1]):  # deterministic sign
            if V[np.argmax(np.abs(V[:, j])), j] < 0:
                V[:, j] = -V[:, j]
        vecs.append(V)
        eig_ops.append(np.diag(w))
    out: List[Term] = []
    for t, (c, ops) in enumerate(terms):
        if t < len(single) and len(ops) == 1 and t in ops and ops[t] is single[t]:
            out.append((c, {t: eig_ops[t]}))  # a mode's own term becomes its eigen operator
        else:
            out.append((c, {d: vecs[d].T @ M @ vecs[d] for d, M in ops.items()}))
    return out, eig_ops


def henon_heiles(D: int = 6, n: int = 10, lam: float = 0.111803, eigenbasis: bool = True) -> HopList:
    """H = sum_i (p_i^2 + q_i^2)/2 + lam sum_{i<D-1} (q_i^2 q_{i+1} - q_{i+1}^3/3).
    One single-mode term per mode (kinetic + harmonic + its -lam/3 q^3 share)
    and one coupling term lam q_i^2 q_{i+1} per neighbouring pair."""
    p2, q1, q2, q3 = ho_p2(n), ho_q_power(n, 1), ho_q_power(n, 2), ho_q_power(n, 3)
    single = []
    for i in range(D):
        h = 0.5 * p2 + 0.5 * q2
        if i >= 1:
            h = h - (lam / 3.0) * q3
        single.append(h)
    terms: List[Term] = [(1.0, {i: single[i]}) for i in range(D)]
    terms += [(lam, {i: q2, i + 1: q1}) for i in range(D - 1)]
    if eigenbasis:
        terms, eig_ops = _to_eigenbasis([n] * D, single, terms)
        return build_hoplist([n] * D, terms, eig_ops)
    return build_hoplist([n] * D, terms)


def coupled_oscillators(D: int, n: int, beta: float = 0.1, eigenbasis: bool = True) -> HopList:
    """The reference's CpOsc system (src/FFPES.f90:166-218): c_i (p_i^2 + q_i^2)
    with c_i = sqrt(i/2)/2 (i 1-based) plus beta q_i q_j for all i < j."""
    p2, q1, q2 = ho_p2(n), ho_q_power(n, 1), ho_q_power(n, 2)
    single = [0.5 * np.sqrt((i + 1) * 0.5) * (p2 + q2) for i in range(D)]
    terms: List[Term] = [(1.0, {i: single[i]}) for i in range(D)]
    terms += [(beta, {i: q1, j: q1}) for i in range(D) for j in range(i + 1, D)]
    if eigenbasis:
        terms, eig_ops = _to_eigenbasis([n] * D, single, terms)
        return build_hoplist([n] * D, terms, eig_ops)
    return build_hoplist([n] * D, terms)


def coupled_oscillators_exact(D: int, beta: float = 0.1) -> np.ndarray:
    """Normal-mode frequencies of the CpOsc Hamiltonian: V = sum c_i q_i^2 +
    beta sum_{i<j} q_i q_j with T = sum c_i p_i^2.  Rescaling to unit mass gives
    eigenvalues of diag(c) + (beta/2)(J - I) ... returned as the list of
    frequencies omega_k such that E = sum_k omega_k (v_k + 1/2)."""
    c = np.array([0.5 * np.sqrt((i + 1) * 0.5) for i in range(D)])
    # H = sum_i c_i p_i^2 + q^T A q with A_ii = c_i, A_ij = beta/2.
    A = np.full((D, D), beta / 2.0)
    np.fill_diagonal(A, c)
    # With p-weights c_i: substitute q_i = sqrt(c_i) x_i -> omega^2 = eig(4 C^1/2 A C^1/2)
    Ch = np.diag(np.sqrt(c))
    return np.sqrt(np.linalg.eigvalsh(4.0 * Ch @ A @ Ch))


def synthetic_qff(D: int, n, seed: int, wmin: float = 200.0, wmax: float = 3200.0, cubic_frac: float = 0.3,
                  cubic_sigma: float = 50.0, quartic_sigma: float = 5.0, eigenbasis: bool = True) -> HopList:
    """Seeded quartic force field in cm^-1 on dimensionless normal coordinates:
    harmonic omega_i (uniform in [wmin, wmax]) as omega_i/2 (p^2 + q^2); cubic
    constants N(0, cubic_sigma) on a random ``cubic_frac`` of index triples;
    semi-diagonal quartic constants N(0, quartic_sigma) on (i,i,j,j).  Each
    constant is divided by the factorials of its mode powers (the reference's
    ``divide`` option, src/FFPES.f90:390-397)."""
    nb, single, terms = qff_terms(D, n, seed, wmin, wmax, cubic_frac, cubic_sigma, quartic_sigma)
    if eigenbasis:
        terms, eig_ops = _to_eigenbasis(nb, single, terms)
        return build_hoplist(nb, terms, eig_ops)
    return build_hoplist(nb, terms)


def qff_terms(D: int, n, seed: int, wmin: float = 200.0, wmax: float = 3200.0, cubic_frac: float = 0.3,
              cubic_sigma: float = 50.0, quartic_sigma: float = 5.0):
    """The terms of synthetic_qff in the primitive harmonic-oscillator basis:
    (nbas, one-mode harmonic operators, [(coef, {mode: operator})]) with the D
    harmonic terms first."""
    rng = np.random.default_rng(seed)
    nb = np.full(D, n, dtype=np.int32) if np.isscalar(n) else np.asarray(n, dtype=np.int32)
    omega = rng.uniform(wmin, wmax, D)
    q = {d: [ho_q_power(int(nb[d]), p) for p in range(5)] for d in range(D)}
    single = [0.5 * omega[d] * (ho_p2(int(nb[d])) + q[d][2]) for d in range(D)]
    terms: List[Term] = [(1.0, {d: single[d]}) for d in range(D)]
    fact = [1, 1, 2, 6, 24]
    for i in range(D):
        for j in range(i, D):
            for k in range(j, D):
                if rng.random() >= cubic_frac:
                    continue
                phi = rng.normal(0.0, cubic_sigma)
                powers: Dict[int, int] = {}
                for m in (i, j, k):
                    powers[m] = powers.get(m, 0) + 1
                for m, p in powers.items():
                    phi /= fact[p]
                terms.append((phi, {m: q[m][p] for m, p in powers.items()}))
    for i in range(D):
        for j in range(i, D):
            phi = rng.normal(0.0, quartic_sigma)
            if i == j:
                terms.append((phi / 24.0, {i: q[i][4]}))
            else:
                terms.append((phi / 4.0, {i: q[i][2], j: q[j][2]}))
    return nb, single, terms


def random_hoplist(nbas: Sequence[int], T: int, seed: int, coupling: int = 2) -> HopList:
    """Random symmetric operators: term t acts on ``coupling`` random modes."""
    rng = np.random.default_rng(seed)
    nbas = np.asarray(nbas, dtype=np.int32)
    D = nbas.size
    terms: List[Term] = []
    for t in range(T):
        modes = rng.choice(D, size=min(coupling, D), replace=False)
        ops = {}
        for d in modes:
            n = int(nbas[d])
            A = rng.normal(size=(n, n)) / np.sqrt(n)
            ops[int(d)] = 0.5 * (A + A.T)
        terms.append((float(rng.uniform(0.5, 1.5)), ops))
    return build_hoplist(nbas, terms)


def dense_hamiltonian(hl: HopList) -> np.ndarray:
    """Full direct-product matrix (small systems only, for checks)."""
    D = hl.ndof
    N = int(np.prod(hl.nbas))
    H = np.zeros((N, N))
    for t in range(hl.nterms):
        M = np.array([[1.0]])
        for d in range(D):
            M = np.kron(M, hl.operator(t, d))
        H += hl.coef[t] * M
    return H


def apply_direct(hl: HopList, x: np.ndarray, ops_cache=None) -> np.ndarray:
    """H x on the full direct-product grid, x shaped (n_0, ..., n_{D-1});
    identity factors are skipped."""
    D = hl.ndof
    out = np.zeros_like(x)
    for t in range(hl.nterms):
        y = x
        for d in range(D):
            M = hl.operator(t, d) if ops_cache is None else ops_cache[t][d]
            if M is None:
                continue
            y = np.moveaxis(np.tensordot(M, y, axes=([1], [d])), 0, d)
        out += hl.coef[t] * y
    return out


def operator_cache(hl: HopList):
    """Dense operators per (term, mode), None where the operator is the identity."""
    cache = []
    for t in range(hl.nterms):
        row = []
        for d in range(hl.ndof):
            M = hl.operator(t, d)
            row.append(None if np.array_equal(M, np.eye(M.shape[0])) else M)
        cache.append(row)
    return cache
