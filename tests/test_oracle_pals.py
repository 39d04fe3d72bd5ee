"""The restated Fortran CPU solver (solver pals at lowmem 4: ALS_POW3,
ALS_ORTHO_2, PRODHV_ALS2, Diagonalize with intertwining, ALS_SUMLCVEC_2).

The reference's GPU path mirrors these routines (src/ALSPow.f90:569 is the
algorithm of POW_ALS, src/ALSUtils.f90:156 of GramSchmidt, :731 of
UPDATES_ALS).  So the two restatements must agree to rounding stage by stage
where the algorithms coincide: the power sweep, the Gram-Schmidt and the
vector updates.  They differ in one place only: the Fortran Rayleigh-Ritz
step reads the upper triangle of the ALS-reduced QHQ (DSYGV 'U') and the GPU
path the lower one.  Known answers cover the rest: exactly representable
products, a numpy eigensolve of the upper triangle, and convergence to exact
spectra.  The plain power solver's routines (solver powr: PRODHV,
PowrRecurse, GRAMORTHO, reductions by reduc_ALS) are checked against dense
products and exactly representable projections.
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import hoplist as H


def dense_block(base, coef, nbas, ranks):
    out, s = [], 0
    for r in ranks:
        out.append(oracle.cp_dense(base[s:s + r], coef[s:s + r], nbas).ravel())
        s += r
    return np.array(out)


def rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def start_block(nbas, rk, nbloc, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.5, 0.5, size=(rk * nbloc, int(np.sum(nbas)))), np.ones(rk * nbloc)


@pytest.mark.parametrize("D,npow", [(4, 3), (3, 2)])
@pytest.mark.parametrize("ishift,esh", [(1, 9.0), (0, 0.0), (-1, 4.0)])
def test_pow3_matches_gpu_algorithm_sweep(ishift, esh, D, npow):
    """With ishift < 0 the GPU path changes the sign of bjk at every mode
    (src/intertw_mvp.cu:437-440), ALS_POW3 at the first mode only
    (src/ALSPow.f90:1265-1269): a mode's factor takes the sign of its own
    step, so each sweep leaves the two vectors (-1)^(D-1) apart.  The
    cycles use ishift = 1."""
    hl = H.henon_heiles(D=D, n=5, lam=0.111803)
    nb, rk, nbloc = hl.nbas, 4, 3
    Q, qc = start_block(nb, rk, nbloc, 1)
    a_b, a_c = oracle.pow_als_block(Q, qc, nb, rk, nbloc, hl, npow, ishift, esh)
    b_b, b_c = oracle.pals_pow3(Q, qc, nb, rk, nbloc, hl, npow, ishift, esh)
    sign = (-1) ** ((D - 1) * npow) if ishift < 0 else 1
    assert rel(dense_block(b_b, b_c, nb, [rk] * nbloc), sign * dense_block(a_b, a_c, nb, [rk] * nbloc)) < 1e-10


def test_pow3_skips_converged_vectors():
    hl = H.random_hoplist([4, 3, 5], 5, seed=4)
    Q, qc = start_block(hl.nbas, 3, 4, 2)
    b, c = oracle.pals_pow3(Q, qc, hl.nbas, 3, 4, hl, 2, 1, 1.0, nconv=2)
    np.testing.assert_array_equal(b[:6], Q[:6])
    np.testing.assert_array_equal(c[:6], qc[:6])
    assert not np.array_equal(c[6:], qc[6:])
    # each swept vector leaves unit norm (the weights are scaled after the last mode)
    for v in (2, 3):
        s = slice(3 * v, 3 * v + 3)
        assert abs(oracle.cp_dot(b[s], c[s], b[s], c[s], hl.nbas) - 1) < 1e-12


def test_ortho2_matches_gpu_algorithm_gram_schmidt():
    hl = H.henon_heiles(D=4, n=5, lam=0.111803)
    nb, rk, nbloc = hl.nbas, 4, 5
    Q, qc = start_block(nb, rk, nbloc, 3)
    Q, qc = oracle.pow_als_block(Q, qc, nb, rk, nbloc, hl, 2, 1, 9.0)
    a_b, a_c = oracle.gram_schmidt(Q, qc, nb, rk, nbloc, 4)
    b_b, b_c = oracle.pals_ortho2(Q, qc, nb, rk, nbloc, 4)
    assert rel(dense_block(b_b, b_c, nb, [rk] * nbloc), dense_block(a_b, a_c, nb, [rk] * nbloc)) < 1e-10


def test_ortho2_ragged_block():
    """ALS_ORTHO_2 keeps a ranks table, so a block may mix ranks: every
    vector leaves with unit norm and the overlaps drop."""
    hl = H.coupled_oscillators(3, 5)
    nb, ranks = hl.nbas, [2, 6, 3, 5]
    rng = np.random.default_rng(7)
    Q = rng.uniform(-0.5, 0.5, size=(sum(ranks), int(nb.sum())))
    qc = np.ones(sum(ranks))
    # a common component makes the start far from orthogonal
    Q[:, :5] += 0.8
    D0 = dense_block(Q, qc, nb, ranks)
    b, c = oracle.pals_ortho2(Q, qc, nb, 0, len(ranks), 12, ranks=ranks)
    D1 = dense_block(b, c, nb, ranks)
    np.testing.assert_allclose(np.einsum("ij,ij->i", D1, D1), 1.0, atol=1e-10)
    off0 = np.abs(np.triu((D0 / np.linalg.norm(D0, axis=1)[:, None]) @ (D0 / np.linalg.norm(D0, axis=1)[:, None]).T,
                          1)).max()
    off1 = np.abs(np.triu(D1 @ D1.T, 1)).max()
    assert off1 < 0.1 * off0


def test_prodhv2_exact_for_one_product_term():
    """With one term acting on one mode, H F has F's rank and the fit
    converges to it."""
    hl = H.random_hoplist([4, 5, 3, 4], 1, seed=9, coupling=1)
    rng = np.random.default_rng(2)
    F = rng.normal(size=(3, int(hl.nbas.sum())))
    fc = rng.uniform(0.5, 1.5, 3)
    b, c = oracle.pals_prodhv2(F, fc, hl.nbas, hl, 200)
    want = H.dense_hamiltonian(hl) @ oracle.cp_dense(F, fc, hl.nbas).ravel()
    got = oracle.cp_dense(b, c, hl.nbas).ravel()
    assert np.linalg.norm(got - want) < 1e-8 * np.linalg.norm(want)


@pytest.mark.parametrize("nitn", [1, 4])
def test_prodhv2_matches_explicit_target_reduction(nitn):
    """PRODHV_ALS2 never forms H F; reduc_ALS on the explicit rT-term H F,
    from the same start, runs the same sweeps with the same update and
    downdate of BB and PS.  Only the penalties differ (1e-10 max c_F against
    1e-15 max c_G)."""
    hl = H.random_hoplist([4, 5, 3, 4], 4, seed=3, coupling=2)
    nb = hl.nbas
    off = np.concatenate([[0], np.cumsum(nb)])
    rng = np.random.default_rng(5)
    F = rng.normal(size=(3, int(nb.sum())))
    fc = rng.uniform(0.5, 1.5, 3)
    gb, gc = [], []
    for t in range(hl.nterms):
        for i in range(3):
            row = np.concatenate([hl.operator(t, d) @ F[i, off[d]:off[d + 1]] for d in range(len(nb))])
            row[:nb[0]] *= hl.coef[t]
            gb.append(row)
            gc.append(fc[i])
    rc, rb = oracle.reduc_als(np.array(gc), np.array(gb), fc, F, nb, nitn)
    b, c = oracle.pals_prodhv2(F, fc, nb, hl, nitn)
    assert rel(oracle.cp_dense(b, c, nb), oracle.cp_dense(rb, rc, nb)) < 1e-8


@pytest.mark.parametrize("ishift", [1, -1])
def test_prodhv2_shift_on_identity_hamiltonian(ishift):
    """H = c I: (H - E) F = (c - E) F exactly, (E - H) F with ishift < 0."""
    nb = [3, 4, 5]
    hl = H.build_hoplist(nb, [(2.5, {})])
    rng = np.random.default_rng(4)
    F = rng.normal(size=(2, sum(nb)))
    fc = np.array([1.0, 0.7])
    E = 4.0
    b, c = oracle.pals_prodhv2(F, fc, nb, hl, 2, ishift=ishift, Eshift=E)
    want = ishift * (2.5 - E) * oracle.cp_dense(F, fc, nb)
    assert rel(oracle.cp_dense(b, c, nb), want) < 1e-9


def test_sumlcvec2_matches_gpu_algorithm_updates():
    hl = H.henon_heiles(D=4, n=5, lam=0.111803)
    nb, rk, nbloc = hl.nbas, 4, 4
    Q, qc = start_block(nb, rk, nbloc, 5)
    Q, qc = oracle.pals_ortho2(Q, qc, nb, rk, nbloc, 3)
    rng = np.random.default_rng(6)
    U = np.linalg.qr(rng.normal(size=(nbloc, nbloc)))[0]
    a_b, a_c = oracle.vector_updates(Q, qc, nb, rk, nbloc, U, 4)
    b_b, b_c = oracle.pals_sumlcvec2(Q, qc, nb, rk, nbloc, U, 4)
    assert rel(dense_block(b_b, b_c, nb, [rk] * nbloc), dense_block(a_b, a_c, nb, [rk] * nbloc)) < 1e-10


def test_diagonalize_reads_upper_triangle():
    """GetQHQ3 + GetOverlaps + DSYGV('U'): the eigenpairs of the matrices
    whose upper triangles hold <Q_j, H Q_i> (H Q_i from PRODHV_ALS2) and
    <Q_j, Q_i>, j >= i."""
    import scipy.linalg
    hl = H.henon_heiles(D=3, n=5, lam=0.111803)
    nb, rk, nbloc, nitn = hl.nbas, 3, 4, 3
    Q, qc = start_block(nb, rk, nbloc, 8)
    Q, qc = oracle.pals_ortho2(Q, qc, nb, rk, nbloc, 4)
    A = np.zeros((nbloc, nbloc))
    S = np.zeros((nbloc, nbloc))
    for i in range(nbloc):
        si = slice(i * rk, (i + 1) * rk)
        hb, hc = oracle.pals_prodhv2(Q[si], qc[si], nb, hl, nitn)
        for j in range(i, nbloc):
            sj = slice(j * rk, (j + 1) * rk)
            A[i, j] = A[j, i] = oracle.cp_dot(Q[sj], qc[sj], hb, hc, nb)
            S[i, j] = S[j, i] = oracle.cp_dot(Q[sj], qc[sj], Q[si], qc[si], nb)
    lam, X = scipy.linalg.eigh(A, S)
    _, _, eig, U = oracle.pals_diagonalize(Q, qc, nb, rk, nbloc, hl, nitn)
    np.testing.assert_allclose(eig, lam, rtol=1e-11, atol=1e-11)
    for m in range(nbloc):
        x = X[:, m] * np.sign(X[np.argmax(np.abs(X[:, m])), m])
        np.testing.assert_allclose(U[:, m], x, atol=1e-9)


def _run(cycle, hl, rk, nbloc, ncyc, npow, nals, seed):
    Q, qc = start_block(hl.nbas, rk, nbloc, seed)
    ex = np.linalg.eigvalsh(H.dense_hamiltonian(hl))
    est = ex[:nbloc] + 0.3
    eig = np.zeros(nbloc)
    for _ in range(ncyc):
        Esh = 0.5 * (2 * est[-1] - est[-2] + ex[-1])
        Q, qc, eig = cycle(Q, qc, hl.nbas, rk, nbloc, hl, eig, npow, nals, True, 1, Esh)
        est = eig
    return eig, ex[:nbloc]


def test_pals_cycle_converges_henon_heiles():
    hl = H.henon_heiles(D=3, n=6, lam=0.111803)
    eig, ex = _run(oracle.pals_cycle, hl, 8, 4, 20, 5, 5, seed=1)
    np.testing.assert_allclose(eig, ex, rtol=1e-5)


def test_pals_cycle_tracks_gpu_algorithm_cycle():
    """Same start, same cycles: the two solvers differ only by the triangle
    of the ALS-reduced QHQ, so their Ritz values stay within the ALS error."""
    hl = H.coupled_oscillators(3, 6)
    e_pals, ex = _run(oracle.pals_cycle, hl, 6, 4, 15, 5, 5, seed=0)
    e_gpu, _ = _run(oracle.intertwine, hl, 6, 4, 15, 5, 5, seed=0)
    np.testing.assert_allclose(e_pals[:-1], ex[:-1], rtol=2e-5)
    np.testing.assert_allclose(e_pals, e_gpu, rtol=1e-3)


# --- the plain power solver (solver powr): PRODHV, PowrRecurse, GRAMORTHO ---

@pytest.mark.parametrize("ishift,E", [(0, 0.0), (1, 3.5), (1, -2.0), (-1, 3.5)])
def test_prodhv_explicit_matches_dense(ishift, E):
    hl = H.random_hoplist([3, 4, 3], 5, seed=12)
    rng = np.random.default_rng(3)
    F = rng.normal(size=(2, int(hl.nbas.sum())))
    fc = rng.uniform(0.5, 1.5, 2)
    gb, gc = oracle.prodhv(F, fc, hl.nbas, hl, ishift, E)
    assert gc.size == 2 * (hl.nterms + (1 if ishift else 0)) and np.all(gc >= 0)
    Hd = H.dense_hamiltonian(hl)
    op = Hd if ishift == 0 else (Hd - E * np.eye(Hd.shape[0])) * (1 if ishift > 0 else -1)
    want = op @ oracle.cp_dense(F, fc, hl.nbas).ravel()
    assert rel(oracle.cp_dense(gb, gc, hl.nbas).ravel(), want) < 1e-13


def test_powr_recurse_on_identity_hamiltonian():
    """H = c I: every step is exactly representable, so the vector keeps its
    direction (the sign of c - E) with unit norm."""
    nb = [3, 4, 3, 2]
    hl = H.build_hoplist(nb, [(1.5, {})])
    rng = np.random.default_rng(8)
    F = rng.normal(size=(3, sum(nb)))
    fc = rng.uniform(0.5, 1.5, 3)
    b, c = oracle.powr_recurse(F, fc, nb, hl, 1, 4.0, 10)
    v0 = oracle.cp_dense(F, fc, nb)
    v1 = oracle.cp_dense(b, c, nb)
    assert rel(v1, -v0 / np.linalg.norm(v0)) < 1e-8


def test_powr_recurse_moves_toward_ground_state():
    hl = H.coupled_oscillators(3, 5)
    ex = np.linalg.eigvalsh(H.dense_hamiltonian(hl))
    rng = np.random.default_rng(2)
    F = rng.uniform(-0.5, 0.5, size=(4, int(hl.nbas.sum())))
    fc = np.ones(4)
    rq0 = oracle.rayleigh_quotient(F, fc, hl.nbas, hl)
    b, c = oracle.powr_recurse(F, fc, hl.nbas, hl, 40, ex[-1] + 1.0, 20)
    rq = oracle.rayleigh_quotient(b, c, hl.nbas, hl)
    assert abs(oracle.cp_dot(b, c, b, c, hl.nbas) - 1) < 1e-12
    assert rq < rq0 and rq - ex[0] < 0.25 * (rq0 - ex[0])


def test_gramortho_exact_projection():
    """Q_0 = x (rank 1), Q_1 = x + y (rank 2), x and y orthogonal products:
    Q_1 - <Q_1, Q_0> Q_0 = y is representable at rank 2, so GRAMORTHO
    returns y / |y|."""
    nb = [3, 4, 3]
    rng = np.random.default_rng(1)
    x = [rng.normal(size=n) for n in nb]
    y = [rng.normal(size=n) for n in nb]
    y[0] = y[0] - x[0] * (y[0] @ x[0]) / (x[0] @ x[0])  # orthogonal in mode 0
    base = np.array([np.concatenate(x), np.concatenate(x), np.concatenate(y)])
    coef = np.array([1.0, 1.0, 0.7])
    b, c = oracle.gramortho(base, coef, nb, 0, 2, 30, ranks=[1, 2])
    yd = oracle.cp_dense(base[2:], coef[2:], nb)
    got = oracle.cp_dense(b[1:], c[1:], nb)
    assert rel(got, yd / np.linalg.norm(yd)) < 1e-8
    xd = oracle.cp_dense(base[:1], coef[:1], nb)
    assert rel(oracle.cp_dense(b[:1], c[:1], nb), xd / np.linalg.norm(xd)) < 1e-13


def test_pgramortho_keeps_leading_vectors():
    hl = H.coupled_oscillators(3, 5)
    nb = hl.nbas
    Q, qc = start_block(nb, 3, 4, 9)
    b0, c0 = oracle.gramortho(Q, qc, nb, 3, 4, 10)
    b1, c1 = oracle.gramortho(b0, c0, nb, 3, 4, 10, k=2)
    np.testing.assert_array_equal(b1[:6], b0[:6])
    np.testing.assert_array_equal(c1[:6], c0[:6])
    D = dense_block(b1, c1, nb, [3] * 4)
    np.testing.assert_allclose(np.einsum("ij,ij->i", D, D), 1.0, atol=1e-12)


def test_pals_edge_cases():
    hl = H.coupled_oscillators(3, 4)
    nb = hl.nbas
    Q, qc = start_block(nb, 3, 1, 4)
    # one vector: the Gram-Schmidt only normalises, the Rayleigh-Ritz value is <Q|H Q>_ALS / <Q|Q>
    b, c, e = oracle.pals_cycle(Q, qc, nb, 3, 1, hl, np.zeros(1), 2, 3, True, 1, 20.0)
    assert e.shape == (1,) and np.isfinite(e[0])
    assert abs(oracle.cp_dot(b, c, b, c, nb) - 1) < 1e-12
    # zero sweeps leave the vectors alone
    b0, c0 = oracle.pals_pow3(Q, qc, nb, 3, 1, hl, 0)
    np.testing.assert_array_equal(b0, Q)
    b0, c0 = oracle.pals_sumlcvec2(Q, qc, nb, 3, 1, np.eye(1), 0)
    np.testing.assert_array_equal(c0, qc)
    with pytest.raises(ValueError):
        oracle.pals_ortho2(Q, qc, nb, 3, 1, 2, ranks=[2])
    with pytest.raises(ValueError):
        oracle.pals_diagonalize(Q, qc, nb, 3, 1, hl, 0)


# --- lowmem 3: the least-memory _3 forms are the same fits as the _2 forms ---

def test_ortho3_matches_ortho2():
    hl = H.henon_heiles(D=4, n=5, lam=0.111803)
    nb, rk, nbloc = hl.nbas, 4, 5
    Q, qc = start_block(nb, rk, nbloc, 13)
    Q, qc = oracle.pals_pow3(Q, qc, nb, rk, nbloc, hl, 2, 1, 9.0)
    a = oracle.pals_ortho2(Q, qc, nb, rk, nbloc, 4)
    b = oracle.pals_ortho2(Q, qc, nb, rk, nbloc, 4, lowmem=3)
    assert rel(dense_block(*b, nb, [rk] * nbloc), dense_block(*a, nb, [rk] * nbloc)) < 1e-10


def test_ortho3_ragged_matches_ortho2():
    hl = H.coupled_oscillators(3, 5)
    nb, ranks = hl.nbas, [2, 6, 3, 5]
    rng = np.random.default_rng(17)
    Q = rng.uniform(-0.5, 0.5, size=(sum(ranks), int(nb.sum())))
    qc = rng.uniform(0.5, 1.0, sum(ranks))
    a = oracle.pals_ortho2(Q, qc, nb, 0, len(ranks), 5, ranks=ranks)
    b = oracle.pals_ortho2(Q, qc, nb, 0, len(ranks), 5, ranks=ranks, lowmem=3)
    assert rel(dense_block(*b, nb, ranks), dense_block(*a, nb, ranks)) < 1e-10


@pytest.mark.parametrize("ishift,E", [(0, 0.0), (1, 6.0), (-1, 6.0)])
def test_prodhv3_matches_prodhv2(ishift, E):
    """The same fit, except the sign with ishift < 0.  PRODHV_ALS2 changes
    the sign of PS and bjk at the first mode (UpdateXPS, DowndateXPS), so
    its targets are (H - E) F at the first mode and (E - H) F at the
    others; BuildbjkDirectX, which PRODHV_ALS3 calls, changes the sign of
    bjk at the first mode only: (E - H) F there, (H - E) F at the others.
    A fit takes the sign of its last mode step's target, so after a sweep
    PRODHV_ALS2 holds (E - H) F, as ishift < 0 asks, and PRODHV_ALS3
    (H - E) F.  The cycles call both with ishift = 0."""
    hl = H.random_hoplist([4, 5, 3, 4], 4, seed=3, coupling=2)
    rng = np.random.default_rng(5)
    F = rng.normal(size=(3, int(hl.nbas.sum())))
    fc = rng.uniform(0.5, 1.5, 3)
    a = oracle.pals_prodhv2(F, fc, hl.nbas, hl, 3, ishift, E)
    b = oracle.pals_prodhv2(F, fc, hl.nbas, hl, 3, ishift, E, lowmem=3)
    sign = -1 if ishift < 0 else 1
    assert rel(oracle.cp_dense(*b, hl.nbas), sign * oracle.cp_dense(*a, hl.nbas)) < 1e-10
    if ishift < 0:
        want = (E * np.eye(int(np.prod(hl.nbas))) - H.dense_hamiltonian(hl)) @ oracle.cp_dense(F, fc, hl.nbas).ravel()
        got = oracle.cp_dense(*a, hl.nbas).ravel()
        assert got @ want > 0.99 * np.linalg.norm(got) * np.linalg.norm(want)


def test_sumlcvec3_matches_sumlcvec2():
    hl = H.henon_heiles(D=4, n=5, lam=0.111803)
    nb, rk, nbloc = hl.nbas, 4, 4
    Q, qc = start_block(nb, rk, nbloc, 19)
    Q, qc = oracle.pals_ortho2(Q, qc, nb, rk, nbloc, 3)
    U = np.linalg.qr(np.random.default_rng(8).normal(size=(nbloc, nbloc)))[0]
    a = oracle.pals_sumlcvec2(Q, qc, nb, rk, nbloc, U, 4)
    b = oracle.pals_sumlcvec2(Q, qc, nb, rk, nbloc, U, 4, lowmem=3)
    assert rel(dense_block(*b, nb, [rk] * nbloc), dense_block(*a, nb, [rk] * nbloc)) < 1e-10


def test_pals_cycle_lowmem3_matches_lowmem4():
    hl = H.coupled_oscillators(3, 6)
    nb, rk, nbloc = hl.nbas, 5, 4
    Q, qc = start_block(nb, rk, nbloc, 23)
    a = oracle.pals_cycle(Q, qc, nb, rk, nbloc, hl, np.zeros(nbloc), 3, 4, True, 1, 25.0)
    b = oracle.pals_cycle(Q, qc, nb, rk, nbloc, hl, np.zeros(nbloc), 3, 4, True, 1, 25.0, lowmem=3)
    np.testing.assert_allclose(b[2], a[2], rtol=1e-10)
    assert rel(dense_block(b[0], b[1], nb, [rk] * nbloc), dense_block(a[0], a[1], nb, [rk] * nbloc)) < 1e-9
    with pytest.raises(ValueError):
        oracle.pals_cycle(Q, qc, nb, rk, nbloc, hl, np.zeros(nbloc), 3, 4, lowmem=5)


# --- lowmem 0-2: the other power steps of ALS_POW_alg ---

@pytest.mark.parametrize("D", [3, 4])
@pytest.mark.parametrize("ishift,esh", [(1, 9.0), (0, 0.0)])
def test_pow_variants(D, ishift, esh):
    """ALS_POW2 keeps BB and PS by update and downdate (UpdateXPS), ALS_POW3
    rebuilds them: the same fit to rounding.  ALS_POW0 (per-mode matrices)
    and ALS_POW1 (update and downdate, or rebuilt for three modes or fewer)
    fit the explicit G with the penalty 1e-15 max c_G instead of 1e-10 max
    c_F: the same as each other to rounding, within 1e-7 of ALS_POW3."""
    hl = H.henon_heiles(D=D, n=5, lam=0.111803)
    nb, rk, nbloc = hl.nbas, 4, 3
    Q, qc = start_block(nb, rk, nbloc, 1)
    res = {lm: dense_block(*oracle.pals_pow(Q, qc, nb, rk, nbloc, hl, 3, ishift, esh, lowmem=lm), nb, [rk] * nbloc)
           for lm in (0, 1, 2, 3)}
    assert rel(res[2], res[3]) < 1e-12
    assert rel(res[0], res[1]) < 1e-12
    assert rel(res[1], res[3]) < 1e-7


def test_pals_cycle_every_lowmem():
    hl = H.coupled_oscillators(3, 6)
    nb, rk, nbloc = hl.nbas, 5, 4
    Q, qc = start_block(nb, rk, nbloc, 23)
    e = {lm: oracle.pals_cycle(Q, qc, nb, rk, nbloc, hl, np.zeros(nbloc), 3, 4, True, 1, 25.0, lowmem=lm)[2]
         for lm in range(5)}
    for lm in (0, 1, 2, 3):
        np.testing.assert_allclose(e[lm], e[4], rtol=1e-7)
