"""Ragged ranks inside the power cycle (intertwineraggedcpp_; the reference
requires equal ranks in a block, src/GPUIterate.f90:152-158).

* Equivalence: a block whose vectors all have rank 5 but are stored with 8
  terms (3 padding terms of random factors) gives, through the ragged entry,
  the same eigenvalues (1e-9 relative) and vectors (1 - |cos| <= 1e-9) as the
  same block stored at rank 5 through intertwinecpp_, in every stage
  (power sweep, Gram-Schmidt, Rayleigh-Ritz, updates).
* Mixed ranks 2..8 in one block: padding weights stay exactly zero, and
  the exact Rayleigh-Ritz values of each returned block (dense H and S of
  the CP vectors) lie above the exact eigenvalues of the small Hamiltonian
  and fall, as a sum, over four cycles.  The cycle's own eigenvalues are
  not a variational bound: the reference builds QHQ(i, j) from
  <Q_j | (H Q_i) reduced to the vector's rank by ALS>
  (src/intertw_mvp.cu:621-630), so a rank-2 vector's Ritz value can fall
  slightly below the exact level; they are only checked to be finite.
"""
import numpy as np
import pytest
import scipy.linalg

import oracle
from mlcp_gb300 import hoplist as H
from mlcp_gb300 import intertwine as IT


def cos_sim(ab, ac, bb, bc, nbas):
    aa = oracle.cp_dot(ab, ac, ab, ac, nbas)
    b2 = oracle.cp_dot(bb, bc, bb, bc, nbas)
    x = oracle.cp_dot(ab, ac, bb, bc, nbas)
    return abs(x) / np.sqrt(aa * b2)


@pytest.mark.gpu
def test_padded_block_equals_unpadded(cuda_device):
    hl = H.random_hoplist([5, 4, 6], 6, seed=31)
    nb = hl.nbas
    nD = int(np.sum(nb))
    B, r, R = 6, 5, 8
    rng = np.random.default_rng(4)
    Q = rng.uniform(-0.5, 0.5, size=(B * r, nD))
    qc = rng.uniform(0.5, 1.0, B * r)
    eig0 = np.arange(B, dtype=float)
    ub, uc, ue = IT.intertwine(Q, qc, nb, r, B, hl, eig0, 3, 4, True, 1, 2.0)
    Qp = rng.uniform(-0.5, 0.5, size=(B * R, nD))
    qcp = np.zeros(B * R)
    for v in range(B):
        Qp[v * R:v * R + r] = Q[v * r:(v + 1) * r]
        qcp[v * R:v * R + r] = qc[v * r:(v + 1) * r]
    pb, pc, pe = IT.intertwine(Qp, qcp, nb, R, B, hl, eig0, 3, 4, True, 1, 2.0, ranks=[r] * B)
    np.testing.assert_allclose(pe, ue, rtol=1e-9)
    for v in range(B):
        assert np.all(pc[v * R + r:(v + 1) * R] == 0.0)
        c = cos_sim(pb[v * R:v * R + r], pc[v * R:v * R + r], ub[v * r:(v + 1) * r], uc[v * r:(v + 1) * r], nb)
        assert 1 - c <= 1e-9, (v, c)


@pytest.mark.gpu
def test_mixed_ranks_stay_ragged_and_variational(cuda_device):
    hl = H.coupled_oscillators(3, 6)
    nb = hl.nbas
    nD = int(np.sum(nb))
    B, R = 7, 8
    ranks = [2, 8, 3, 5, 8, 4, 6]
    rng = np.random.default_rng(5)
    Q = rng.uniform(-0.5, 0.5, size=(B * R, nD))
    qc = np.ones(B * R)
    Hd = H.dense_hamiltonian(hl)
    spectrum = np.sort(np.linalg.eigvalsh(Hd))
    exact = spectrum[:B]

    def ritz(Q, qc):
        # exact Rayleigh-Ritz values of the block, each vector at its own rank
        Qd = np.array([oracle.cp_dense(Q[v * R:v * R + ranks[v]], qc[v * R:v * R + ranks[v]], nb)
                       for v in range(B)])
        return scipy.linalg.eigh(Qd @ Hd @ Qd.T, Qd @ Qd.T, eigvals_only=True)

    eig = np.arange(B, dtype=float) + 1.0
    sums = []
    for cyc in range(4):
        esh = IT.block_shift(eig, spectrum[-1])  # GetBlockShift: the power steps favour the lowest states
        Q, qc, eig = IT.intertwine(Q, qc, nb, R, B, hl, eig, 4, 4, True, 1, esh, ranks=ranks)
        for v in range(B):
            assert np.all(qc[v * R + ranks[v]:(v + 1) * R] == 0.0)
        assert np.all(np.isfinite(eig))
        lam = ritz(Q, qc)
        assert np.all(lam >= exact - 1e-9 * np.abs(exact)), (lam, exact)
        sums.append(float(np.sum(lam)))
    assert sums[-1] < sums[0], sums


@pytest.mark.gpu
def test_ragged_block_matches_fortran_cpu_solver(cuda_device):
    """The Fortran host's CPU solver keeps a ranks table (ALS_ORTHO_2,
    src/ALSUtils.f90:180-200), so it runs a ragged block as it is.  The GPU's
    ragged cycle without update (power sweeps, then Gram-Schmidt) against its
    restated ALS_POW3 and ALS_ORTHO_2 on the same block, stored compactly:
    every vector agrees to 1e-8 (largest entry of the dense difference over
    the largest entry).  With update the two read opposite triangles of the
    ALS-reduced QHQ (DSYGV 'U' against the GPU path's lower one), which
    moves low-rank Ritz values by up to several percent, so that stage is
    left to the variational checks above."""
    hl = H.coupled_oscillators(3, 6)
    nb = hl.nbas
    nD = int(np.sum(nb))
    B, R = 6, 7
    ranks = [3, 7, 2, 5, 4, 6]
    rng = np.random.default_rng(12)
    Q = rng.uniform(-0.5, 0.5, size=(B * R, nD))
    qc = rng.uniform(0.5, 1.0, B * R)
    live = np.concatenate([np.arange(v * R, v * R + ranks[v]) for v in range(B)])
    eig0 = np.arange(B, dtype=float) + 1.0
    esh = 14.0
    gb, gc, ge = IT.intertwine(Q, qc, nb, R, B, hl, eig0, 3, 4, False, 1, esh, ranks=ranks)
    np.testing.assert_array_equal(ge, eig0)
    cb, cc = oracle.pals_pow3(Q[live], qc[live], nb, 0, B, hl, 3, 1, esh, ranks=ranks)
    cb, cc = oracle.pals_ortho2(cb, cc, nb, 0, B, 4, ranks=ranks)
    s = 0
    for v in range(B):
        g = oracle.cp_dense(gb[v * R:v * R + ranks[v]], gc[v * R:v * R + ranks[v]], nb)
        c = oracle.cp_dense(cb[s:s + ranks[v]], cc[s:s + ranks[v]], nb)
        s += ranks[v]
        assert np.abs(g - c).max() <= 1e-8 * np.abs(c).max(), v
