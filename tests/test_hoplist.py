"""Operator-list layout (reference src/hoplist.h:2-7, src/ModeH.f90:909-1068)
and harmonic-oscillator matrix elements."""
import numpy as np

from mlcp_gb300 import hoplist as H


def test_pack_index_rule():
    n = 5
    M = np.arange(n * n, dtype=float).reshape(n, n)
    M = M + M.T
    v = H.pack(M)
    for c in range(n):
        for r in range(c + 1):
            assert v[r + c * (c + 1) // 2] == M[r, c]
    np.testing.assert_array_equal(H.unpack(v, n), M)


def test_ho_matrix_elements():
    q2 = H.ho_q_power(6, 2)
    q4 = H.ho_q_power(6, 4)
    p2 = H.ho_p2(6)
    assert abs(q2[0, 0] - 0.5) < 1e-15 and abs(q4[0, 0] - 0.75) < 1e-15
    assert abs(q2[0, 2] - np.sqrt(2) / 2) < 1e-15 and abs(p2[0, 2] + np.sqrt(2) / 2) < 1e-15
    # <i|(p^2+q^2)/2|j> = (i + 1/2) delta_ij
    np.testing.assert_allclose(0.5 * (p2 + q2)[:5, :5], np.diag(np.arange(5) + 0.5), atol=1e-14)
    q1 = H.ho_q_power(8, 1)
    np.testing.assert_allclose((q1 @ q1 @ q1)[:5, :5], H.ho_q_power(5, 3), atol=1e-13)


def test_hoplist_reference_layout():
    hl = H.henon_heiles(D=4, n=5)
    D = 4
    T = hl.nterms
    assert hl.opid.size == T * D
    # the first D operators are the identities, the next D the eigen operators
    for d in range(D):
        np.testing.assert_array_equal(H.unpack(hl.mat[hl.mptr[d] - 1:hl.mptr[d] - 1 + 15], 5), np.eye(5))
    # single-mode term d uses the eigen operator of mode d, identity elsewhere
    for d in range(D):
        for e in range(D):
            expect = D + d + 1 if e == d else e + 1
            assert hl.opid[d * D + e] == expect
    # mptr is 1-based and increasing in steps of the packed sizes
    assert hl.mptr[0] == 1
    assert np.all(np.diff(hl.mptr) == 15)
    assert hl.mat.size == (hl.mptr[-1] - 1) + 15


def test_apply_direct_matches_dense():
    hl = H.random_hoplist([3, 4, 2], 5, seed=1)
    rng = np.random.default_rng(0)
    x = rng.normal(size=(3, 4, 2))
    y = H.apply_direct(hl, x)
    Hd = H.dense_hamiltonian(hl)
    np.testing.assert_allclose(y.ravel(), Hd @ x.ravel(), atol=1e-12)


def test_qff_is_seeded_and_symmetric():
    a = H.synthetic_qff(4, 5, seed=3)
    b = H.synthetic_qff(4, 5, seed=3)
    np.testing.assert_array_equal(a.mat, b.mat)
    np.testing.assert_array_equal(a.opid, b.opid)
    Hd = H.dense_hamiltonian(a)
    np.testing.assert_allclose(Hd, Hd.T, atol=1e-9)
