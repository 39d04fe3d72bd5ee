"""The CPU oracle against mathematical known answers (the reference has no
golden data for this path, so these pin the restatement instead):

* exactly representable reductions are reproduced by ALS;
* the generalised eigensolver agrees with a dense numpy solution;
* full CP inner products agree with dense tensor contractions;
* repeated intertwined power cycles converge to the exact eigenvalues of
  small Hamiltonians (dense diagonalisation, analytic normal modes).
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import hoplist as H


def dense_cp(base, coef, nbas):
    offs = np.concatenate([[0], np.cumsum(nbas)])
    out = 0.0
    for r in range(len(coef)):
        t = np.array([coef[r]])
        for d in range(len(nbas)):
            t = np.multiply.outer(t, base[r, offs[d]:offs[d + 1]])
        out = out + t
    return out


def test_cp_dot_matches_dense():
    rng = np.random.default_rng(1)
    nbas = [3, 4, 2, 5]
    nD = sum(nbas)
    vb, vc = rng.normal(size=(4, nD)), rng.uniform(0.1, 1, 4)
    wb, wc = rng.normal(size=(3, nD)), rng.uniform(0.1, 1, 3)
    ref = np.sum(dense_cp(vb, vc, nbas) * dense_cp(wb, wc, nbas))
    assert abs(oracle.cp_dot(vb, vc, wb, wc, nbas) - ref) < 1e-12 * max(1, abs(ref))


def test_als_reproduces_exact_target():
    rng = np.random.default_rng(0)
    nbas = [4, 5, 3, 6]
    nD = sum(nbas)
    rF = 3
    Ft = rng.normal(size=(rF, nD))
    ct = rng.uniform(0.5, 2, rF)
    base = np.vstack([rng.normal(size=(rF, nD)), Ft, Ft])
    coef = np.concatenate([np.ones(rF), 0.5 * ct, 0.5 * ct])
    c, b = oracle.als(coef, base, nbas, rF, 2 * rF, 200)
    G = dense_cp(base[rF:], coef[rF:], nbas)
    F = dense_cp(b, c, nbas)
    assert np.linalg.norm(F - G) / np.linalg.norm(G) < 1e-6


def test_als_monotone_residual():
    """ALS never increases ||F - G|| from one sweep to the next (up to the
    tiny penalty)."""
    rng = np.random.default_rng(4)
    nbas = [5, 4, 6]
    nD = sum(nbas)
    G = rng.normal(size=(12, nD))
    cg = rng.uniform(0.1, 1, 12)
    F0 = G[:3].copy()
    base = np.vstack([F0, G])
    coef = np.concatenate([cg[:3], cg])
    Gd = dense_cp(G, cg, nbas)
    prev = np.inf
    for s in range(1, 8):
        c, b = oracle.als(coef, base, nbas, 3, 12, s)
        r = np.linalg.norm(dense_cp(b, c, nbas) - Gd)
        assert r <= prev * (1 + 1e-9)
        prev = r


def test_oracle_als_drift_under_fp32_rhs():
    """How far an FP64 ALS trajectory moves when nothing changes but its
    right-hand sides being rounded to FP32 before each solve: tiny after one
    sweep, about 1e-6 in relative residual and 6e-5 in distance after four
    sweeps on this slowly converging rank-9 fit of a rank-150 target.  The GPU
    parity tests bound multi-sweep drift from this measurement."""
    from mlcp_gb300 import workloads

    def cp_dot(ab, ac, bb, bc):
        return oracle.cp_dot(ab, ac, bb, bc, batch.nbas)

    def rel(ac, ab, bc, bb):
        aa, bbv, x = cp_dot(ab, ac, ab, ac), cp_dot(bb, bc, bb, bc), cp_dot(ab, ac, bb, bc)
        return np.sqrt(max(aa + bbv - 2 * x, 0.0) / bbv)

    batch = workloads.als_batch(2, 5, 16, 9, 150, seed=13)
    c0, b0 = batch.vector(1)
    pc, pb, rGp = oracle.pad_target(c0, b0, 9, 150)
    drift = {}
    try:
        for nals in (1, 4):
            oracle.set_rhs_fp32(False)
            oc, ob = oracle.als(pc, pb, batch.nbas, 9, rGp, nals)
            oracle.set_rhs_fp32(True)
            qc, qb = oracle.als(pc, pb, batch.nbas, 9, rGp, nals)
            res = abs(rel(oc, ob, c0[9:], b0[9:]) - rel(qc, qb, c0[9:], b0[9:]))
            drift[nals] = (res, rel(qc, qb, oc, ob))
    finally:
        oracle.set_rhs_fp32(False)
    assert drift[1][0] < 1e-8 and drift[1][1] < 1e-6
    assert drift[4][0] > 5e-7 and drift[4][1] > 2e-5


def test_sygv_matches_dense():
    rng = np.random.default_rng(2)
    n = 7
    A = rng.normal(size=(n, n))
    A = A + A.T
    B = rng.normal(size=(n, n))
    B = B @ B.T + n * np.eye(n)
    w, X, info = oracle.sygv(A, B)
    assert info == 0
    L = np.linalg.cholesky(B)
    Li = np.linalg.inv(L)
    wr = np.linalg.eigvalsh(Li @ A @ Li.T)
    np.testing.assert_allclose(w, wr, atol=1e-12)
    np.testing.assert_allclose(X.T @ B @ X, np.eye(n), atol=1e-12)
    np.testing.assert_allclose(A @ X, B @ X * w, atol=1e-10)
    for j in range(n):  # sign convention: largest-magnitude entry positive
        assert X[np.argmax(np.abs(X[:, j])), j] > 0


def _run_cycles(hl, rk, nbloc, ncyc, npow, nals, seed):
    rng = np.random.default_rng(seed)
    D = hl.ndof
    nD = int(hl.nbas.sum())
    Q = rng.uniform(-0.5, 0.5, size=(rk * nbloc, nD))
    qc = np.ones(rk * nbloc)
    Hd = H.dense_hamiltonian(hl)
    ex = np.linalg.eigvalsh(Hd)
    est = ex[:nbloc] + 0.3
    eig = np.zeros(nbloc)
    for _ in range(ncyc):
        a = 2 * est[-1] - est[-2]
        Esh = 0.5 * (a + ex[-1])
        Q, qc, eig = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig, npow=npow, nals=nals, update=True,
                                       ishift=1, Eshift=Esh)
        est = eig
    return eig, ex[:nbloc]


def test_intertwine_coupled_oscillators_converge():
    hl = H.coupled_oscillators(3, 6)
    eig, ex = _run_cycles(hl, 6, 4, 15, 5, 5, seed=0)
    # the top vector of a block converges slowest under block power iteration
    np.testing.assert_allclose(eig[:-1], ex[:-1], rtol=2e-5)
    np.testing.assert_allclose(eig[-1], ex[-1], rtol=1e-3)


def test_coupled_oscillators_analytic_ground_state():
    """The dense spectrum of CpOsc matches its normal-mode frequencies
    (checks the HO operator matrices and the HopList assembly)."""
    D = 3
    hl = H.coupled_oscillators(D, 12)
    ex = np.linalg.eigvalsh(H.dense_hamiltonian(hl))
    w = H.coupled_oscillators_exact(D)
    assert abs(ex[0] - 0.5 * w.sum()) < 1e-8
    assert abs(ex[1] - (0.5 * w.sum() + w.min())) < 1e-6


def test_intertwine_henon_heiles_converges():
    hl = H.henon_heiles(D=3, n=6, lam=0.111803)
    eig, ex = _run_cycles(hl, 8, 4, 20, 5, 5, seed=1)
    np.testing.assert_allclose(eig, ex, rtol=1e-5)


def test_intertwine_no_update_only_orthogonalises():
    hl = H.random_hoplist([4, 3, 5], 6, seed=3)
    rng = np.random.default_rng(5)
    rk, nbloc = 3, 3
    Q = rng.normal(size=(rk * nbloc, 12))
    qc = np.ones(rk * nbloc)
    eig = np.array([1.0, 2.0, 3.0])
    Q2, qc2, eig2 = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig, npow=2, nals=20, update=False,
                                      ishift=1, Eshift=1.5)
    np.testing.assert_array_equal(eig2, eig)
    nb = hl.nbas
    # vectors are approximately orthonormal after the ALS-guided Gram-Schmidt
    for i in range(nbloc):
        vi = slice(i * rk, (i + 1) * rk)
        nii = oracle.cp_dot(Q2[vi], qc2[vi], Q2[vi], qc2[vi], nb)
        assert abs(nii - 1) < 1e-6
        for j in range(i):
            vj = slice(j * rk, (j + 1) * rk)
            assert abs(oracle.cp_dot(Q2[vi], qc2[vi], Q2[vj], qc2[vj], nb)) < 5e-2


def test_pow_als_zero_iterations_is_identity():
    hl = H.random_hoplist([3, 4], 3, seed=2)
    rng = np.random.default_rng(0)
    Q = rng.normal(size=(4, 7))
    qc = np.ones(4)
    b, c = oracle.pow_als_block(Q, qc, hl.nbas, 2, 2, hl, npow=0)
    np.testing.assert_array_equal(b, Q)
    np.testing.assert_array_equal(c, qc)


@pytest.mark.parametrize("make", [lambda: H.henon_heiles(D=3, n=5, lam=0.111803),
                                  lambda: H.coupled_oscillators(3, 5),
                                  lambda: H.random_hoplist([4, 3, 5], 6, seed=7)])
def test_rayleigh_quotient_matches_dense(make):
    """RayleighQuotient2 restatement = v^T H v / v^T v with the dense
    Hamiltonian and the dense vector."""
    hl = make()
    Hd = H.dense_hamiltonian(hl)
    rng = np.random.default_rng(3)
    rk, nD = 4, int(hl.nbas.sum())
    b, c = rng.normal(size=(rk, nD)), rng.uniform(0.3, 1.5, rk)
    v = dense_cp(b, c, list(hl.nbas)).reshape(-1)
    want = v @ Hd @ v / (v @ v)
    got = oracle.rayleigh_quotient(b, c, hl.nbas, hl)
    assert abs(got - want) <= 1e-12 * abs(want)


def test_qhq_diag_skips_converged_vectors():
    hl = H.random_hoplist([4, 5, 3], 5, seed=4)
    rng = np.random.default_rng(9)
    rk, nbloc, nD = 3, 5, int(hl.nbas.sum())
    Q, qc = rng.normal(size=(rk * nbloc, nD)), rng.uniform(0.5, 1.0, rk * nbloc)
    out = oracle.qhq_diag(Q, qc, hl.nbas, rk, nbloc, hl, nconv=2, qhqd=np.full(nbloc, -7.0))
    assert np.all(out[:2] == -7.0)
    for i in range(2, nbloc):
        s = slice(i * rk, (i + 1) * rk)
        assert out[i] == oracle.rayleigh_quotient(Q[s], qc[s], hl.nbas, hl)


def test_sort_vecs_semantics():
    """SortVecs: increasing |eigv - Eref|, vectors follow, nconv cut back."""
    rk, nD = 2, 3
    eig = np.array([1.0, 5.0, 2.5, 0.2])
    Q = np.arange(4 * rk * nD, dtype=float).reshape(4 * rk, nD)
    qc = np.arange(4 * rk, dtype=float)
    b, c, e, nconv = oracle.sort_vecs(Q, qc, rk, eig, 3, 2.0)
    assert list(e) == [2.5, 1.0, 0.2, 5.0]
    assert np.array_equal(b[:rk], Q[2 * rk:3 * rk]) and np.array_equal(c[rk:2 * rk], qc[:rk])
    assert nconv == 0
    _, _, e2, nconv2 = oracle.sort_vecs(Q, qc, rk, np.array([0.1, 0.2, 0.3, 0.4]), 3, 0.0)
    assert list(e2) == [0.1, 0.2, 0.3, 0.4] and nconv2 == 3


@pytest.mark.parametrize("make", [lambda: H.henon_heiles(D=3, n=5, lam=0.111803),
                                  lambda: H.coupled_oscillators(3, 5)])
def test_spectral_range_brackets_and_converges(make):
    """GetSpectralRange restatement: the unpadded bounds are Rayleigh
    quotients, so they lie in [E_min, E_max]; after enough rounds they reach
    both ends of the dense spectrum (to the accuracy a rank-4 power iteration
    reaches: 1e-4 of the spectral width at the top, 1e-3 at the bottom, where
    the shifted iteration converges more slowly)."""
    hl = make()
    ex = np.linalg.eigvalsh(H.dense_hamiltonian(hl))
    b, c = oracle.spectral_start(hl.nbas, 4, seed=1)
    _, _, bd = oracle.spectral_range(b, c, hl.nbas, 4, hl, 5, 20)
    pad = 0.001 * (bd[1] - bd[0]) / 1.002
    lo, hi = bd[0] + pad, bd[1] - pad
    assert ex[0] - 1e-9 <= lo <= hi <= ex[-1] + 1e-9
    width = ex[-1] - ex[0]
    assert abs(hi - ex[-1]) < 1e-4 * width
    assert abs(lo - ex[0]) < 1e-3 * width


def test_update_opermat_matches_dense():
    """UpdateOperMat restatement = Q X_m Q^T with dense vectors and X acting
    on mode m (identity elsewhere), packed upper-triangular."""
    rng = np.random.default_rng(0)
    nbas, rk, nbloc = [3, 4, 2], 2, 3
    nD = sum(nbas)
    Q, qc = rng.normal(size=(nbloc * rk, nD)), rng.uniform(0.5, 1.0, nbloc * rk)
    Qd = np.array([dense_cp(Q[i * rk:(i + 1) * rk], qc[i * rk:(i + 1) * rk], nbas).reshape(-1)
                   for i in range(nbloc)])
    for imode in (1, 2, 3):
        n = nbas[imode - 1]
        X = rng.normal(size=(n, n))
        X = X + X.T
        packed = np.array([X[i, j] for j in range(n) for i in range(j + 1)])
        out = oracle.update_opermat(imode, Q, qc, nbas, rk, nbloc, packed)[0]
        eyes = [np.eye(m) for m in nbas]
        eyes[imode - 1] = X
        Xf = np.kron(np.kron(eyes[0], eyes[1]), eyes[2])
        want = Qd @ Xf @ Qd.T
        assert np.max(np.abs(oracle.unpack_sym(out, nbloc) - want)) <= 1e-12 * np.max(np.abs(want))


def test_reduc_svd_restatement():
    """reduc_SVD restatement: an exact rank-3 input comes back as the same
    matrix with 3 terms (the zero singular values fall below redtol * s_1);
    truncation to rF terms leaves the Eckart-Young error; the factors are
    orthonormal; a zero vector keeps min(nr, nc, rF) zero-weight terms."""
    rng = np.random.default_rng(3)
    nbas = [7, 5]
    b3, c3 = rng.normal(size=(3, 12)), rng.uniform(0.5, 2.0, 3)
    b = np.concatenate([b3, b3[:2]])
    c = np.concatenate([c3, [0.5, -0.25]])  # rank 3, five terms
    A = oracle.cp2d_dense(b, c, nbas)
    ob, oc = oracle.reduc_svd(b, c, nbas, 10)
    assert oc.size == 3
    np.testing.assert_allclose(oracle.cp2d_dense(ob, oc, nbas), A, atol=1e-13 * np.abs(A).max())
    np.testing.assert_allclose(ob[:, :7] @ ob[:, :7].T, np.eye(3), atol=1e-14)
    np.testing.assert_allclose(ob[:, 7:] @ ob[:, 7:].T, np.eye(3), atol=1e-14)
    s = np.linalg.svd(A, compute_uv=False)
    ob2, oc2 = oracle.reduc_svd(b, c, nbas, 2)
    err = np.linalg.norm(oracle.cp2d_dense(ob2, oc2, nbas) - A)
    assert abs(err - s[2]) < 1e-12 * s[0]
    ob0, oc0 = oracle.reduc_svd(b, np.zeros(5), nbas, 4)
    assert oc0.size == 4 and not np.any(oc0)


@pytest.mark.parametrize("make", [lambda: H.coupled_oscillators(2, 8),
                                  lambda: H.random_hoplist([9, 7], 5, seed=4)])
def test_spectral_range_2mode_brackets(make):
    """Two-mode GetSpectralRange restatement (PowrRecurse with SVD): the
    unpadded bounds are Rayleigh quotients inside [E_min, E_max] and reach
    both ends of the dense spectrum (1e-6 of the width: the SVD reduction is
    exact up to the rank cut, unlike ALS)."""
    hl = make()
    ex = np.linalg.eigvalsh(H.dense_hamiltonian(hl))
    _, bd = oracle.spectral_range_2mode(hl.nbas, 8, hl, 10, 12)
    pad = 0.001 * (bd[1] - bd[0]) / 1.002
    lo, hi = bd[0] + pad, bd[1] - pad
    assert ex[0] - 1e-9 <= lo <= hi <= ex[-1] + 1e-9
    width = ex[-1] - ex[0]
    assert abs(hi - ex[-1]) < 1e-6 * width
    assert abs(lo - ex[0]) < 1e-6 * width


def test_diagonalize_dense_restatement():
    """Diagonalize restatement: a block of all the product functions of a
    two-mode node (the solver's diag case) gives the exact spectrum, and the
    SVD-reduced eigenfunctions are the exact eigenvectors (rank <= 3 = the
    smaller mode, so the reduction is exact)."""
    hl = H.random_hoplist([4, 3], 5, seed=9)
    nb = [4, 3]
    rk, B = 3, 12
    base = np.full((B * rk, 7), 0.0)
    coef = np.zeros(B * rk)
    for a in range(4):
        for b in range(3):
            i = a * 3 + b
            base[i * rk, a] = 1.0
            base[i * rk, 4 + b] = 1.0
            coef[i * rk] = 1.0
    vecs, _, lam, U = oracle.diagonalize_dense(base, coef, nb, rk, B, hl)
    Hd = H.dense_hamiltonian(hl)
    ex, X = np.linalg.eigh(Hd)
    np.testing.assert_allclose(lam, ex, rtol=1e-12, atol=1e-12)
    for m in range(B):
        v = oracle.cp_dense(*vecs[m], nb)
        assert abs(abs(v @ X[:, m]) - 1.0) < 1e-10


@pytest.mark.parametrize("ishift,esh", [(1, 6.0), (-1, 1.5)])
def test_pow_sweep_is_scale_free(ishift, esh):
    """The in-place power sweep fits (H - E) F and renormalises the weights at
    the end of each sweep, so scaling H and E by a power of two (2^40) leaves
    its output bit-identical in FP64.  The GPU sweep's weight rescaling relies
    on exactly this invariance (its test compares H with 2^40 H)."""
    hl = H.henon_heiles(D=4, n=6)
    big = H.HopList(nbas=hl.nbas, opid=hl.opid, mptr=hl.mptr, coef=hl.coef * 2.0 ** 40, mat=hl.mat)
    rk, nbloc = 6, 3
    rng = np.random.default_rng(5)
    Q = rng.uniform(-0.5, 0.5, size=(rk * nbloc, int(np.sum(hl.nbas))))
    qc = np.ones(rk * nbloc)
    a = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, np.zeros(nbloc), 3, 0, False, ishift, esh)
    b = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, big, np.zeros(nbloc), 3, 0, False, ishift, esh * 2.0 ** 40)
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def _reduc_als_numpy(gc, gb, fc, fb, nbas, nitn):
    """Independent numpy restatement of reduc_ALS (src/REDUCTIONML.f90:593-731)
    with every product rebuilt from scratch at each mode step (the update
    scheme of the C restatement only reorders these products)."""
    offs = np.concatenate([[0], np.cumsum(nbas)])
    fc, fb = fc.copy(), fb.copy()
    pen = gc.max() * 1e-15
    D = len(nbas)
    for _ in range(nitn):
        for k in range(D):
            sl = slice(offs[k], offs[k + 1])
            BB = np.ones((fc.size, fc.size))
            PS = np.ones((gc.size, fc.size))
            for d in range(D):
                if d == k:
                    continue
                s = slice(offs[d], offs[d + 1])
                BB *= fb[:, s] @ fb[:, s].T
                PS *= gb[:, s] @ fb[:, s].T
            BB += pen * np.eye(fc.size)
            b = (PS * gc[:, None]).T @ gb[:, sl]
            X = np.linalg.solve(BB, b)
            nrm = np.sqrt(np.abs(np.sum(X * X, axis=1)))
            fc = nrm
            fb[:, sl] = X / nrm[:, None]
    return fc, fb


@pytest.mark.parametrize("D,nbas,rF,rG,nitn", [(3, [4, 5, 3], 3, 17, 4), (5, [4, 6, 5, 3, 7], 4, 30, 5),
                                                (6, [5] * 6, 6, 40, 3)])
def test_reduc_als_matches_independent_restatement(D, nbas, rF, rG, nitn):
    """reduc_ALS (the reference's CPU ALS, the timed reference CPU path)
    against an independent numpy form that rebuilds every product: the same
    reduced vector to 1e-7 as a function.  Five and six modes take the
    update/downdate branch of the running products (each step divides out
    and multiplies back one mode's dots, whose rounding the ALS iteration
    carries and amplifies: 2e-8 measured after five sweeps), three modes the
    rebuild branch (below 1e-12)."""
    rng = np.random.default_rng(D)
    nD = int(np.sum(nbas))
    gb = rng.normal(size=(rG, nD))
    gc = rng.uniform(0.1, 1.0, rG)
    fb = gb[:rF].copy() + 0.1 * rng.normal(size=(rF, nD))
    fc = np.ones(rF)
    oc, ob = oracle.reduc_als(gc, gb, fc, fb, nbas, nitn)
    nc, nb_ = _reduc_als_numpy(gc, gb, fc, fb, np.array(nbas), nitn)
    aa = oracle.cp_dot(ob, oc, ob, oc, nbas)
    bb = oracle.cp_dot(nb_, nc, nb_, nc, nbas)
    ab = oracle.cp_dot(ob, oc, nb_, nc, nbas)
    assert np.sqrt(max(aa + bb - 2 * ab, 0.0) / bb) < (1e-7 if D > 3 else 1e-12)
    # the fit improves on the start
    gg = oracle.cp_dot(gb, gc, gb, gc, nbas)

    def res(c, b):
        return np.sqrt(max(oracle.cp_dot(b, c, b, c, nbas) + gg - 2 * oracle.cp_dot(b, c, gb, gc, nbas), 0) / gg)
    assert res(oc, ob) < res(fc, fb)
