"""Two-mode SVD reduction (reducsvdcpp_, reference reduc_SVDa/b,
src/REDUCTIONML.f90:296-392) on the GPU against the oracle's restatement
(CP2DtoMat, LAPACK SVD through numpy, the reference's truncation rule).

The GPU forms A in FP64 and runs the Jacobi sweeps in double-word (about
48-bit) arithmetic.  Singular vectors are unique only up to the sign of
each (u_i, v_i) pair, so results are compared as the kept rank, the
singular values (1e-12 of s_1), the reduced vector as a matrix (1e-12 of
its largest entry) and the orthonormality of each mode's factors (1e-12).
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import intertwine as IT


def make_batch(rng, nvec, rG, nbas, low_rank=None):
    nD = sum(nbas)
    base = rng.normal(size=(nvec, rG, nD))
    coef = rng.uniform(0.2, 2.0, size=(nvec, rG))
    if low_rank is not None:  # repeat the first low_rank terms: exact rank low_rank
        for k in range(low_rank, rG):
            base[:, k] = base[:, k % low_rank]
    return base, coef


def check(gb, gc, gr, base, coef, nbas, rF, redtol=1e-12):
    nr = nbas[0]
    for v in range(base.shape[0]):
        ob, oc = oracle.reduc_svd(base[v], coef[v], nbas, rF, redtol)
        k = oc.size
        assert gr[v] == k
        assert not np.any(gc[v, k:]) and not np.any(gb[v, k:])
        np.testing.assert_allclose(gc[v, :k], oc, rtol=0, atol=1e-12 * max(oc[0], 1e-300))
        G = oracle.cp2d_dense(gb[v, :k], gc[v, :k], nbas)
        O = oracle.cp2d_dense(ob, oc, nbas)
        assert np.abs(G - O).max() <= 1e-12 * max(np.abs(O).max(), 1e-300)
        U, W = gb[v, :k, :nr], gb[v, :k, nr:]
        np.testing.assert_allclose(U @ U.T, np.eye(k), atol=1e-12)
        np.testing.assert_allclose(W @ W.T, np.eye(k), atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("nbas,rG,rF,nvec", [([12, 9], 30, 6, 5), ([9, 12], 30, 6, 5), ([64, 64], 200, 16, 3),
                                             ([33, 17], 8, 20, 4), ([1, 5], 3, 2, 2), ([6, 1], 4, 3, 2),
                                             ([100, 120], 150, 40, 2), ([130, 150], 160, 30, 2)])
def test_reduc_svd_matches_oracle(nbas, rG, rF, nvec, cuda_device):
    """Full-rank inputs: square, both orientations (nr > nc, nr < nc), a
    one-function mode, rF above the attainable rank, a 100 x 120 case
    (120 x 100 after the transpose; 176 KB of shared memory) and a
    130 x 150 case whose Jacobi sweeps run in global memory."""
    rng = np.random.default_rng(rG + rF)
    base, coef = make_batch(rng, nvec, rG, nbas)
    gb, gc, gr = IT.reduc_svd(base.reshape(-1, sum(nbas)), coef.ravel(), nbas, rG, rF)
    check(gb, gc, gr, base, coef, nbas, rF)


@pytest.mark.gpu
def test_reduc_svd_rank_cut(cuda_device):
    """Exact rank-5 inputs of 24 terms: ncomp = 5 (the other singular values
    are rounding noise far below redtol * s_1), so at most 5 terms remain."""
    rng = np.random.default_rng(9)
    nbas = [20, 16]
    base, coef = make_batch(rng, 4, 24, nbas, low_rank=5)
    gb, gc, gr = IT.reduc_svd(base.reshape(-1, 36), coef.ravel(), nbas, 24, 10)
    assert list(gr) == [5] * 4
    check(gb, gc, gr, base, coef, nbas, 10)


@pytest.mark.gpu
def test_reduc_svd_zero_vector(cuda_device):
    """A zero input (s_1 = 0, so no value falls below the cut): the reference
    keeps min(nr, nc, rF) terms of weight zero; the matrix stays zero."""
    nbas = [7, 4]
    base = np.random.default_rng(1).normal(size=(6, 11))
    gb, gc, gr = IT.reduc_svd(base, np.zeros(6), nbas, 6, 5)
    assert gr[0] == 4 and not np.any(gc)
    assert not np.any(oracle.cp2d_dense(gb[0], gc[0], nbas))


@pytest.mark.gpu
def test_reduc_svd_rejects_bad_sizes(cuda_device):
    with pytest.raises(Exception, match="reducsvdcpp_"):
        IT.reduc_svd(np.zeros((2, 600)), np.ones(2), [300, 300], 2, 4)
