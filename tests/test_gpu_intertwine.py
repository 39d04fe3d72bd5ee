"""GPU intertwined power cycle (intertwinecpp_ through the C ABI) against the
FP64 oracle.

Both sides use the reference's FP64-build penalty rule (1e-10 max c,
src/als.cu:248-267) in every stage; the oracle is the reference's FP64
algorithm (pinned against the reference library in test_gpu_reference.py).

Tolerances (double-word power sweeps, Gram-Schmidt and updates, FP64
Rayleigh-Ritz): eigenvalues agree to 1e-6 relative; each output vector
agrees with the oracle's as a function, |<a,b>| / (|a| |b|) >= 1 - 1e-6
(sign-insensitive: the eigenvector sign convention is fixed identically on
both sides, but a vector's factors may carry compensating signs).
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import hoplist as H
from mlcp_gb300 import intertwine as IT

EIG_RTOL = 1e-6
COS_TOL = 1e-6


def cos_sim(ab, ac, bb, bc, nbas):
    aa = oracle.cp_dot(ab, ac, ab, ac, nbas)
    bbv = oracle.cp_dot(bb, bc, bb, bc, nbas)
    x = oracle.cp_dot(ab, ac, bb, bc, nbas)
    return abs(x) / np.sqrt(aa * bbv)


def start_block(nbas, rk, nbloc, seed):
    rng = np.random.default_rng(seed)
    Q = rng.uniform(-0.5, 0.5, size=(rk * nbloc, int(np.sum(nbas))))
    qc = np.ones(rk * nbloc)
    return Q, qc


def compare_blocks(gb, gc, ob, oc, nbas, rk, nbloc, tol=COS_TOL):
    worst = 1.0
    for i in range(nbloc):
        s = slice(i * rk, (i + 1) * rk)
        worst = min(worst, cos_sim(gb[s], gc[s], ob[s], oc[s], nbas))
    assert 1 - worst <= tol, worst


CASES = [
    # (hoplist factory, rk, nbloc, npow, nals, update, ishift, Eshift)
    (lambda: H.random_hoplist([4, 5, 3], 6, seed=3), 3, 4, 3, 4, True, 1, 2.0),
    (lambda: H.coupled_oscillators(3, 6), 5, 4, 4, 4, True, 1, 4.0),
    (lambda: H.henon_heiles(D=4, n=6), 6, 5, 3, 3, True, 1, 6.0),
    (lambda: H.random_hoplist([6, 4, 5, 3], 9, seed=8, coupling=3), 4, 3, 2, 3, False, -1, 1.5),
    (lambda: H.random_hoplist([5, 7], 4, seed=2), 3, 3, 3, 0, False, 0, 0.0),
    # 34 vectors: a 16-CTA Gram-Schmidt cluster, up to 3 earlier vectors per CTA
    (lambda: H.random_hoplist([4, 3, 5], 5, seed=11), 3, 34, 1, 2, False, 1, 3.0),
    # rank 40: the Gram-Schmidt overlaps and earlier vectors do not fit in
    # shared memory (global scratch); solves by the four-warp refinement
    (lambda: H.random_hoplist([5, 4, 6, 3], 5, seed=21), 40, 20, 1, 2, False, 1, 3.0),
    # rank 24 (one right-hand-side column per warp) and a mode of 20 basis
    # functions (more columns than the register solve takes)
    (lambda: H.random_hoplist([20, 5, 6], 5, seed=22), 24, 6, 2, 3, True, 1, 3.0),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(CASES)))
def test_cycle_matches_oracle(case, cuda_device):
    make, rk, nbloc, npow, nals, update, ishift, esh = CASES[case]
    hl = make()
    Q, qc = start_block(hl.nbas, rk, nbloc, seed=case)
    eig0 = np.arange(nbloc, dtype=float)
    gb, gc, ge = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, npow, nals, update, ishift, esh)
    ob, oc, oe = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, npow, nals, update, ishift, esh)
    if update:
        np.testing.assert_allclose(ge, oe, rtol=EIG_RTOL, atol=1e-12)
    else:
        np.testing.assert_array_equal(ge, eig0)
    compare_blocks(gb, gc, ob, oc, hl.nbas, rk, nbloc)


@pytest.mark.gpu
def test_cycles_converge_to_exact_spectrum(cuda_device):
    """Known answer: repeated GPU cycles reproduce the lowest eigenvalues of a
    small Henon-Heiles Hamiltonian from dense diagonalisation.  The tolerance
    (3e-5 relative) is the converged accuracy of a rank-8 representation of
    the near-degenerate pair at 2.4886/2.4904 under the FP32-build penalty;
    the oracle under the same rule converges to the same values."""
    hl = H.henon_heiles(D=3, n=6, lam=0.111803)
    ex = np.linalg.eigvalsh(H.dense_hamiltonian(hl))
    rk, nbloc = 8, 4
    Q, qc = start_block(hl.nbas, rk, nbloc, seed=1)
    est = ex[:nbloc] + 0.3
    eig = np.zeros(nbloc)
    for _ in range(20):
        esh = IT.block_shift(est, ex[-1])
        Q, qc, eig = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig, 5, 5, True, 1, esh)
        est = eig
    np.testing.assert_allclose(eig, ex[:nbloc], rtol=3e-5)


@pytest.mark.gpu
def test_cycle_rejects_bad_operator_index(cuda_device):
    hl = H.random_hoplist([4, 3], 3, seed=1)
    bad = H.HopList(nbas=hl.nbas, opid=hl.opid.copy(), mptr=hl.mptr, coef=hl.coef, mat=hl.mat)
    bad.opid[2] = hl.mptr.size + 5
    Q, qc = start_block(hl.nbas, 2, 2, seed=0)
    with pytest.raises(Exception, match="opid"):
        IT.intertwine(Q, qc, hl.nbas, 2, 2, bad, np.zeros(2), 2, 2, True, 1, 1.0)


@pytest.mark.gpu
def test_cycle_rejects_block_above_rayleigh_ritz_limit(cuda_device):
    """The one-CTA Rayleigh-Ritz solve takes at most 160 vectors; a larger
    block with update = T is an error return (checked before any device work)."""
    hl = H.random_hoplist([4, 3], 3, seed=1)
    Q, qc = start_block(hl.nbas, 2, 161, seed=0)
    with pytest.raises(Exception, match="160 vectors"):
        IT.intertwine(Q, qc, hl.nbas, 2, 161, hl, np.zeros(161), 1, 1, True, 1, 1.0)


QHQ_CASES = [
    # (hoplist factory, rk, nbloc, nconv)
    (lambda: H.henon_heiles(D=3, n=5), 4, 6, 0),
    (lambda: H.coupled_oscillators(3, 6), 1, 2, 0),
    (lambda: H.random_hoplist([5, 4, 6, 3], 5, seed=21), 40, 3, 1),
    (lambda: H.henon_heiles(D=6, n=10, lam=0.111803), 16, 40, 5),
]


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(QHQ_CASES)))
def test_qhq_diag_matches_oracle(case, cuda_device):
    """getqhqdiagcpp_ (GetQHQdiag / RayleighQuotient2) against the oracle:
    both FP64, so only the summation order differs (1e-11 relative)."""
    make, rk, nbloc, nconv = QHQ_CASES[case]
    hl = make()
    Q, qc = start_block(hl.nbas, rk, nbloc, seed=20 + case)
    init = np.full(nbloc, -3.0)
    g = IT.qhq_diag(Q, qc, hl.nbas, rk, nbloc, hl, nconv, init)
    o = oracle.qhq_diag(Q, qc, hl.nbas, rk, nbloc, hl, nconv, init)
    assert np.all(g[:nconv] == -3.0)
    np.testing.assert_allclose(g, o, rtol=1e-11)


@pytest.mark.gpu
def test_update_false_path_matches_oracle(cuda_device):
    """The reference host's update = F step (src/Solver.f90:498-504): a cycle
    without Rayleigh-Ritz, Rayleigh quotients of the block, then SortVecs
    about the lower spectral bound.  Same tolerances as the cycle tests."""
    hl = H.henon_heiles(D=4, n=6)
    rk, nbloc = 6, 5
    Q, qc = start_block(hl.nbas, rk, nbloc, seed=31)
    eig0 = np.arange(nbloc, dtype=float)
    gb, gc, _ = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, 3, 3, False, 1, 6.0)
    ob, oc, _ = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, 3, 3, False, 1, 6.0)
    ge = IT.qhq_diag(gb, gc, hl.nbas, rk, nbloc, hl)
    oe = oracle.qhq_diag(ob, oc, hl.nbas, rk, nbloc, hl)
    np.testing.assert_allclose(ge, oe, rtol=EIG_RTOL)
    gb, gc, ge, gn = IT.sort_vecs(gb, gc, hl.nbas, rk, ge, 2, 2.0)
    ob, oc, oe, on = oracle.sort_vecs(ob, oc, rk, oe, 2, 2.0)
    assert gn == on
    np.testing.assert_allclose(ge, oe, rtol=EIG_RTOL)
    compare_blocks(gb, gc, ob, oc, hl.nbas, rk, nbloc)


@pytest.mark.gpu
@pytest.mark.parametrize("ncyc", [0, 1, 6])
def test_spectral_range_matches_oracle(ncyc, cuda_device):
    """getspectralrangecpp_ against the oracle from the same starting vectors."""
    hl = H.henon_heiles(D=4, n=6)
    b, c = oracle.spectral_start(hl.nbas, 5, seed=2)
    gb, gc, gbd = IT.spectral_range(b, c, hl.nbas, 5, hl, 4, ncyc)
    ob, oc, obd = oracle.spectral_range(b, c, hl.nbas, 5, hl, 4, ncyc)
    np.testing.assert_allclose(gbd, obd, rtol=1e-6)
    compare_blocks(gb, gc, ob, oc, hl.nbas, 5, 2, tol=1e-5)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [("random", [9, 7], 6, 4, 3), ("random", [7, 11], 5, 3, 2),
                                  ("oscillators", [8, 8], 8, 10, 5), ("random", [40, 33], 12, 3, 2)])
def test_spectral_range_two_modes_matches_oracle(case, cuda_device):
    """Two-mode getspectralrangecpp_ (PowrRecurse: exact H v in FP64, SVD
    reduction with double-word Jacobi sweeps, NORMCOEF) against the oracle's
    FP64 restatement: bounds to 1e-10
    relative, each final vector as a matrix to 1e-9 of its largest entry
    (the SVD's sign freedom cancels in U S V^T).  [7, 11] takes the
    transposed orientation (nr < nc); [40, 33] a 40 x 33 SVD per step."""
    kind, nbas, rk, npow, ncyc = case
    hl = H.coupled_oscillators(2, nbas[0]) if kind == "oscillators" else H.random_hoplist(nbas, 5, seed=rk)
    b, c = oracle.spectral_start(hl.nbas, rk)
    gb, gc, gbd = IT.spectral_range(b, c, hl.nbas, rk, hl, npow, ncyc)
    vecs, obd = oracle.spectral_range_2mode(hl.nbas, rk, hl, npow, ncyc)
    np.testing.assert_allclose(gbd, obd, rtol=1e-10)
    for j in range(2):
        G = oracle.cp2d_dense(gb[j * rk:(j + 1) * rk], gc[j * rk:(j + 1) * rk], hl.nbas)
        O = oracle.cp2d_dense(*vecs[j], hl.nbas)
        assert np.abs(G - O).max() <= 1e-9 * np.abs(O).max()


@pytest.mark.gpu
def test_spectral_range_rejects_one_mode(cuda_device):
    hl = H.random_hoplist([5], 4, seed=2)
    b, c = oracle.spectral_start(hl.nbas, 3)
    with pytest.raises(Exception, match="two modes"):
        IT.spectral_range(b, c, hl.nbas, 3, hl, 2, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("imode,rk,nbloc,nx", [(1, 4, 6, 1), (3, 16, 40, 3), (2, 5, 9, 20)])
def test_update_opermat_matches_oracle(imode, rk, nbloc, nx, cuda_device):
    """updateopermatcpp_ (UpdateOperMat for nx operators at once) against the
    oracle; both FP64 (1e-12 of the largest entry).  20 operators take two
    passes of the pair kernel."""
    rng = np.random.default_rng(imode + nx)
    nbas = [5, 6, 4, 3]
    n = nbas[imode - 1]
    Q, qc = start_block(nbas, rk, nbloc, seed=imode)
    xm = []
    for _ in range(nx):
        X = rng.normal(size=(n, n))
        X = X + X.T
        xm.append([X[i, j] for j in range(n) for i in range(j + 1)])
    xm = np.array(xm)
    g = IT.update_opermat(imode, Q, qc, nbas, rk, nbloc, xm)
    o = oracle.update_opermat(imode, Q, qc, nbas, rk, nbloc, xm)
    assert np.max(np.abs(g - o)) <= 1e-12 * np.max(np.abs(o))


def product_block(nbas, rk):
    """Every product function of a two-mode node as a rank-1 vector padded to
    rank rk with zero weights (the solver's diag case: nev = nr * nc)."""
    nr, nc = nbas
    B = nr * nc
    base = np.zeros((B * rk, nr + nc))
    coef = np.zeros(B * rk)
    for a in range(nr):
        for b in range(nc):
            i = a * nc + b
            base[i * rk, a] = 1.0
            base[i * rk, nr + b] = 1.0
            coef[i * rk] = 1.0
    return base, coef, B


def dense_cos(gb, gc, ob, oc, nbas):
    g, o = oracle.cp_dense(gb, gc, nbas), oracle.cp_dense(ob, oc, nbas)
    return abs(g @ o) / np.sqrt((g @ g) * (o @ o))


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["diag", "block"])
def test_diagonalize_two_modes_matches_oracle(case, cuda_device):
    """diagonalizecpp_ on two modes (exact <Q|H|Q> and <Q|Q> in FP64, the
    generalised eigenproblem, SVD-reduced eigenfunctions) against the dense
    restatement: eigenvalues to 1e-9 relative, each new vector to
    1 - |cos| <= 1e-9.  "diag": all 20 product functions of a 5 x 4 node (the
    exact spectrum); "block": 6 random rank-3 vectors on 7 x 6."""
    if case == "diag":
        nbas, rk = [5, 4], 4
        hl = H.random_hoplist(nbas, 6, seed=31)
        base, coef, B = product_block(nbas, rk)
    else:
        nbas, rk, B = [7, 6], 3, 6
        hl = H.random_hoplist(nbas, 5, seed=32)
        base, coef = start_block(nbas, rk, B, seed=5)
    gb, gc, ge = IT.diagonalize(base, coef, nbas, rk, B, hl, 0)
    vecs, _, lam, _ = oracle.diagonalize_dense(base, coef, nbas, rk, B, hl)
    np.testing.assert_allclose(ge, lam, rtol=1e-9, atol=1e-9 * np.abs(lam).max())
    for m in range(B):
        s = slice(m * rk, (m + 1) * rk)
        assert 1 - dense_cos(gb[s], gc[s], *vecs[m], nbas) <= 1e-9, m
    if case == "diag":
        np.testing.assert_allclose(ge, np.linalg.eigvalsh(H.dense_hamiltonian(hl)), rtol=1e-9,
                                   atol=1e-9 * np.abs(lam).max())


@pytest.mark.gpu
@pytest.mark.parametrize("nals", [0, 3])
def test_diagonalize_three_modes_matches_oracle(nals, cuda_device):
    """diagonalizecpp_ on three modes: eigenvalues of the exact block problem
    to 1e-9 relative; with nals > 0 the vectors updated by ALS from the old
    ones (FP32 contractions, as the cycle's updates: 1 - |cos| <= 1e-6
    against the restated update with the dense solve's eigenvectors), with
    nals = 0 left unchanged."""
    nbas, rk, B = [4, 5, 3], 3, 5
    hl = H.random_hoplist(nbas, 6, seed=33)
    base, coef = start_block(nbas, rk, B, seed=6)
    gb, gc, ge = IT.diagonalize(base, coef, nbas, rk, B, hl, nals)
    ob, oc, lam, _ = oracle.diagonalize_dense(base, coef, nbas, rk, B, hl, nals)
    np.testing.assert_allclose(ge, lam, rtol=1e-9, atol=1e-9 * np.abs(lam).max())
    if nals == 0:
        np.testing.assert_array_equal(gb, base)
        np.testing.assert_array_equal(gc, coef)
    else:
        compare_blocks(gb, gc, ob, oc, nbas, rk, B)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [1, 3, 7])
def test_cycle_graph_replay_matches_eager_launches(case, cuda_device):
    """The cycle replayed from its captured CUDA graph gives bit-identical
    blocks and eigenvalues to the same cycle launched kernel by kernel, over
    three cycles that change the shift (a device input of the graph) and
    interleave another shape (which recaptures)."""
    from mlcp_gb300 import _lib
    L = _lib.load()
    make, rk, nbloc, npow, nals, update, ishift, esh = CASES[case]
    hl = make()
    other = H.random_hoplist([4, 5, 3], 6, seed=3)
    Q0, qc0 = start_block(hl.nbas, rk, nbloc, seed=40 + case)
    Qo, qco = start_block(other.nbas, 3, 4, seed=99)
    outs = {}
    for graph in (0, 1):
        L.mlcp_gb300_set_cycle_graph(graph)
        Q, qc, eig = Q0.copy(), qc0.copy(), np.arange(nbloc, dtype=float)
        res = []
        for cyc in range(3):
            Q, qc, eig = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig, npow, nals, update, ishift,
                                       esh + 0.5 * cyc)
            IT.intertwine(Qo, qco, other.nbas, 3, 4, other, np.arange(4.0), 2, 2, True, 1, 2.0)
            res.append((Q.copy(), qc.copy(), eig.copy()))
        outs[graph] = res
    L.mlcp_gb300_set_cycle_graph(1)
    for (a, b) in zip(outs[0], outs[1]):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [5, 6])
@pytest.mark.parametrize("groups", [2, 3])
def test_gram_schmidt_over_several_clusters(case, groups, cuda_device, monkeypatch):
    """The Gram-Schmidt spread over several 16-CTA clusters (a cooperative
    launch whose cluster leaders exchange their partial right-hand sides
    through global memory each mode step; the library picks it for blocks
    whose arrays do not fit in shared memory) against one cluster and the
    oracle: the same cycle to the oracle tolerances, and to 1e-9 of the
    one-cluster result (only the order of the partial sums differs)."""
    from mlcp_gb300 import _lib
    L = _lib.load()
    L.mlcp_gb300_set_cycle_graph(0)  # the cluster count is read at launch time
    try:
        make, rk, nbloc, npow, nals, update, ishift, esh = CASES[case]
        hl = make()
        Q, qc = start_block(hl.nbas, rk, nbloc, seed=case)
        eig0 = np.arange(nbloc, dtype=float)
        res = {}
        for g in (1, groups):
            monkeypatch.setenv("MLCP_GB300_GS_GROUPS", str(g))
            res[g] = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, npow, nals, update, ishift, esh)
        ob, oc, oe = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, npow, nals, update, ishift, esh)
        gb, gc, ge = res[groups]
        compare_blocks(gb, gc, ob, oc, hl.nbas, rk, nbloc)
        compare_blocks(gb, gc, res[1][0], res[1][1], hl.nbas, rk, nbloc, tol=1e-9)
    finally:
        L.mlcp_gb300_set_cycle_graph(1)


@pytest.mark.gpu
def test_gram_schmidt_cluster_search(cuda_device):
    """The first cycle of a block shape times one Gram-Schmidt sweep for each
    candidate cluster size (16, 12 and 8 CTAs) on a scratch copy of the block
    and keeps the fastest; the autotune report lists the trials.  The cycle
    with the search off (the 16-CTA rule) agrees with it to 1e-9 (the cluster
    size only changes the order of the partial sums)."""
    from mlcp_gb300 import _lib
    L = _lib.load()
    hl = H.henon_heiles(D=4, n=6, lam=0.111803)
    rk, nbloc = 5, 20
    Q, qc = start_block(hl.nbas, rk, nbloc, seed=21)
    eig0 = np.arange(nbloc, dtype=float)
    tb, tc, te = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, 2, 3, True, 1, 30.0)
    lines = [ln for ln in _lib.autotune_report().splitlines() if ln.startswith(f"gs nbloc={nbloc} R={rk} ")]
    assert len(lines) == 1, _lib.autotune_report()
    chosen = int(lines[0].split("cluster ")[1].split(";")[0])
    trials = dict((int(a), float(b[:-2])) for a, b in (t.split("=") for t in lines[0].split(";")[1].split()))
    assert sorted(trials) == [8, 12, 16] and chosen in trials
    assert trials[chosen] == min(trials.values())
    L.mlcp_gb300_set_autotune(0)
    try:
        rb, rc, re_ = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, 2, 3, True, 1, 30.0)
    finally:
        L.mlcp_gb300_set_autotune(1)
    np.testing.assert_allclose(te, re_, rtol=1e-9)
    compare_blocks(tb, tc, rb, rc, hl.nbas, rk, nbloc, tol=1e-9)
