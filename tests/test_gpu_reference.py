"""Parity against the reference's own FP64 CUDA library (the plain FP64 GPU
form), run on the same GPU in a child process (oracle/ref_build.py builds it
from the reference's sources, oracle/ref_run.py serves its alscpp_ and
intertwinecpp_).

Two kinds of check:

* The oracle is pinned to the reference: the C restatement gives the same
  ALS residuals to 1e-12 relative and the same vectors to 1e-7 as functions,
  and the same cycle eigenvalues to 1e-8 relative (both FP64; they differ
  only in summation order and in cuSOLVER's LU against the oracle's).
* The GPU path against the reference:
  - ALS (explicit target, alscpp_): on the benchmark shape (30 modes of 12,
    3200 -> 20 terms, 10 sweeps) the relative residuals ||F - G|| / ||G||
    agree to 1e-6 relative (measured 9e-16).  On the small fits, stopped
    after 3-10 sweeps far from convergence, the FP32 contractions bound the
    agreement: |r_gpu - r_ref| <= SMALL_RES_RTOL = 1e-5 of r_ref or
    ABS_RES_TOL = 6e-8.  Measured 1.4e-6 to 4.3e-6 relative over runs: the
    summation order of the right-hand sides follows the launch shape the
    autotuner picks (cluster size, ring depth), and an unconverged
    trajectory carries each step's FP32 rounding (~1e-7 of ||G||, plus the
    running products' multiply/divide updates) into the next; the FP64
    oracle with only its right-hand sides rounded to FP32 moves by 1.7e-6
    after four sweeps (tests/test_oracle.py).  The vectors agree to 2e-5 as
    functions.
  - The power cycle (intertwinecpp_): from a block the solver has brought
    near convergence, one cycle's eigenvalues agree to CYCLE_EIG_RTOL = 1e-7
    relative (the Henon-Heiles parity bound; measured 4e-11) and each vector
    to 1 - |cos| <= 1e-7.  Along three solver-loop cycles the reference
    shadows the GPU (one cycle from the GPU's block at every cycle), to the
    same bounds.  Left free-running, the two trajectories separate (the block
    is not fully converged and each side feeds its own block back): the
    reference amplifies a 1e-12 perturbation of its own starting weights to
    6e-10 in three cycles, and the GPU's 4e-11 first-cycle difference to
    ~2e-6.  From the solver's
    product-function guess, whose 1e-12-weight augmentation terms make the
    first normal equations as ill-conditioned as the penalty allows, the
    double-word stages drift from FP64 by a few 1e-6 in the first cycles
    (bound 2e-5).

Every case feeds both sides identical explicit inputs (no random starts).
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import als, workloads

ABS_RES_TOL = 6e-8
REL_RES_TOL = 1e-6
SMALL_RES_RTOL = 1e-5
GPU_VEC_TOL = 2e-5
CYCLE_EIG_RTOL = 1e-7
CYCLE_COS_TOL = 1e-7


@pytest.fixture(scope="module")
def ref():
    if not oracle.reference_staged():
        pytest.skip("the reference's CUDA sources are not staged (oracle/ref_build.py needs the reference tree)")
    assert oracle.reference_built(), "reference sources are staged but oracle/_ref/libmlcpref.so is not built"
    r = oracle.Reference(timeout=1500)
    yield r
    r.close()


def rel_residual(fc, fb, gc, gb, nbas):
    ff = oracle.cp_dot(fb, fc, fb, fc, nbas)
    gg = oracle.cp_dot(gb, gc, gb, gc, nbas)
    fg = oracle.cp_dot(fb, fc, gb, gc, nbas)
    return np.sqrt(max(ff + gg - 2 * fg, 0.0) / gg)


def rel_distance(ac, ab, bc, bb, nbas):
    aa = oracle.cp_dot(ab, ac, ab, ac, nbas)
    bbv = oracle.cp_dot(bb, bc, bb, bc, nbas)
    x = oracle.cp_dot(ab, ac, bb, bc, nbas)
    return np.sqrt(max(aa + bbv - 2 * x, 0.0) / bbv)


def cos_sim(ab, ac, bb, bc, nbas):
    aa = oracle.cp_dot(ab, ac, ab, ac, nbas)
    bbv = oracle.cp_dot(bb, bc, bb, bc, nbas)
    x = oracle.cp_dot(ab, ac, bb, bc, nbas)
    return abs(x) / np.sqrt(aa * bbv)


ALS_CASES = [
    # (D, nbas, rF, rG, nals); rG a multiple of rF, as the reference walks the target in blocks of rF
    (4, [4, 5, 3, 6], 3, 12, 5),
    (6, 12, 8, 64, 10),
    (5, [20, 12, 40, 7, 17], 9, 153, 4),
    (3, [6, 5, 4], 16, 256, 3),
    (2, [10, 14], 5, 60, 6),
    (30, 12, 20, 200, 3),  # more modes than the rank (the reference's nbas sizing fix)
]


def gpu_reduce(batch, nals, dev):
    import torch
    c = torch.from_numpy(batch.coef.copy()).to(dev)
    b = torch.from_numpy(batch.base.copy()).to(dev)
    st = torch.zeros(batch.nvec, dtype=torch.int32, device=dev)
    als.reduce_batched(c, b, batch.nbas, batch.rF, batch.rG, batch.term_off, nals, status=st)
    torch.cuda.synchronize()
    assert not st.any()
    return c.cpu().numpy(), b.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ALS_CASES)
def test_als_oracle_and_gpu_match_reference(case, ref, cuda_device):
    D, n, rF, rG, nals = case
    batch = workloads.als_batch(1, D, n, rF, rG, seed=5)
    c0, b0 = batch.vector(0)
    rc, rb, _ = ref.als(c0[None], b0[None], batch.nbas, rF, rG, nals)
    rc, rb = rc[0], rb[0]
    oc, ob = oracle.als(c0, b0, batch.nbas, rF, rG, nals)
    gc, gb = gpu_reduce(batch, nals, cuda_device)
    gc, gb = gc[:rF], gb[:rF]
    tgt = (c0[rF:], b0[rF:])
    r_ref = rel_residual(rc, rb, *tgt, batch.nbas)
    r_orc = rel_residual(oc, ob, *tgt, batch.nbas)
    r_gpu = rel_residual(gc, gb, *tgt, batch.nbas)
    # the oracle is the reference's algorithm
    assert abs(r_orc - r_ref) <= 1e-12 * r_ref, (r_orc, r_ref)
    assert rel_distance(oc, ob, rc, rb, batch.nbas) <= 1e-7
    # the GPU path
    assert abs(r_gpu - r_ref) <= max(SMALL_RES_RTOL * r_ref, ABS_RES_TOL), (r_gpu, r_ref)
    assert rel_distance(gc, gb, rc, rb, batch.nbas) <= GPU_VEC_TOL


@pytest.mark.gpu
def test_als_benchmark_shape_matches_reference(ref, cuda_device):
    """Four vectors of the benchmark batch (64 x 30 modes of 12, 3200 -> 20,
    10 sweeps, the seeded batch bench.py times), reduced by the GPU inside
    the whole batch and one by one by the reference."""
    batch = workloads.als_batch(64, 30, 12, 20, 3200)
    gc, gb = gpu_reduce(batch, 10, cuda_device)
    vs = [0, 1, 2, 3]
    cs = np.stack([batch.vector(v)[0] for v in vs])
    bs = np.stack([batch.vector(v)[1] for v in vs])
    rc, rb, _ = ref.als(cs, bs, batch.nbas, 20, 3200, 10)
    for k, v in enumerate(vs):
        c0, b0 = batch.vector(v)
        t = int(batch.term_off[v])
        tgt = (c0[20:], b0[20:])
        r_ref = rel_residual(rc[k], rb[k], *tgt, batch.nbas)
        r_gpu = rel_residual(gc[t:t + 20], gb[t:t + 20], *tgt, batch.nbas)
        assert abs(r_gpu - r_ref) <= REL_RES_TOL * r_ref, (v, r_gpu, r_ref)
        assert rel_distance(gc[t:t + 20], gb[t:t + 20], rc[k], rb[k], batch.nbas) <= GPU_VEC_TOL


def bench_cycle_inputs():
    """The power-cycle workload bench.py times: Henon-Heiles D=6, n=10,
    lambda = 0.111803, rank 16, a seeded random block of 40 vectors."""
    from mlcp_gb300 import hoplist as H
    hl = H.henon_heiles(D=6, n=10, lam=0.111803)
    rng = np.random.default_rng(20261203)
    Q = rng.uniform(-0.5, 0.5, size=(16 * 40, 60))
    qc = np.ones(16 * 40)
    eig0 = 3.0 + np.sort(np.concatenate([[0], np.ones(6), 2 * np.ones(21), 3 * np.ones(56)]))[:40]
    esh = 0.5 * (2 * eig0[-1] - eig0[-2] + (3.0 + 9 * 6))
    return hl, Q, qc, eig0, esh


@pytest.mark.gpu
def test_cycle_oracle_matches_reference(ref):
    """One intertwined cycle (npow = nals = 10, update on) from a random block:
    the oracle, on the reference's FP64 penalty rule in every stage, gives the
    reference's eigenvalues and vectors."""
    hl, Q, qc, eig0, esh = bench_cycle_inputs()
    rbq, rcq, re, _ = ref.intertwine(Q, qc, hl.nbas, 16, 40, hl, eig0, 10, 10, True, 1, esh)
    ob, oc, oe = oracle.intertwine(Q, qc, hl.nbas, 16, 40, hl, eig0, 10, 10, True, 1, esh)
    assert np.max(np.abs(oe - re) / np.abs(re)) <= 1e-8
    worst = min(cos_sim(ob[i * 16:(i + 1) * 16], oc[i * 16:(i + 1) * 16], rbq[i * 16:(i + 1) * 16],
                        rcq[i * 16:(i + 1) * 16], hl.nbas) for i in range(40))
    assert 1 - worst <= 1e-8, worst


def converged_block(ncycle=40):
    """The bench cycle's block after ncycle solver cycles on the GPU (from the
    product-function guess), with the spectral bounds of that run."""
    from mlcp_gb300 import hoplist as H
    from mlcp_gb300 import solver
    hl = H.henon_heiles(D=6, n=10, lam=0.111803)
    base, coef, eigv, bounds, _ = solver.solve(hl, 40, 16, ncycle, 10, 10)
    return hl, base, coef, eigv, bounds


@pytest.mark.gpu
def test_cycle_gpu_matches_reference_near_convergence(ref, cuda_device):
    """From a block the solver has brought near convergence, one GPU cycle and
    one reference cycle on identical inputs: eigenvalues to 1e-7 relative,
    vectors to 1 - |cos| <= 1e-7."""
    from mlcp_gb300 import intertwine as IT
    hl, base, coef, eigv, bounds = converged_block()
    esh = IT.block_shift(eigv, bounds[1])
    rb, rc, re, _ = ref.intertwine(base, coef, hl.nbas, 16, 40, hl, eigv, 10, 10, True, 1, esh)
    gb, gc, ge = IT.intertwine(base, coef, hl.nbas, 16, 40, hl, eigv, 10, 10, True, 1, esh)
    rel = np.abs(ge - re) / np.abs(re)
    assert rel.max() <= CYCLE_EIG_RTOL, rel.max()
    worst = min(cos_sim(gb[i * 16:(i + 1) * 16], gc[i * 16:(i + 1) * 16], rb[i * 16:(i + 1) * 16],
                        rc[i * 16:(i + 1) * 16], hl.nbas) for i in range(40))
    assert 1 - worst <= CYCLE_COS_TOL, worst


@pytest.mark.gpu
def test_solver_loop_tracks_reference_near_convergence(ref, cuda_device):
    """The solver loop (block shift, one cycle, repeat) from the same
    near-converged block, three cycles.  At every cycle the reference runs
    one cycle from the GPU's current block and shift (a shadow of the GPU's
    trajectory): its eigenvalues and vectors agree with the GPU's to
    CYCLE_EIG_RTOL = 1e-7 and CYCLE_COS_TOL.  The free-running trajectories
    (each side feeding back its own block) are printed, not bounded: on this
    unconverged block the reference itself amplifies a 1e-12 perturbation of
    its starting weights to 6e-10 in three cycles, and the GPU's first-cycle
    difference (4e-11) grows the same way to ~2e-6."""
    from mlcp_gb300 import intertwine as IT
    hl, base, coef, eigv, bounds = converged_block()
    gb, gc, ge = base.copy(), coef.copy(), eigv.copy()
    rb, rc, re = base.copy(), coef.copy(), eigv.copy()
    for cyc in range(3):
        esh = IT.block_shift(ge, bounds[1])
        sb, sc, se, _ = ref.intertwine(gb, gc, hl.nbas, 16, 40, hl, ge, 10, 10, True, 1, esh)
        gb, gc, ge = IT.intertwine(gb, gc, hl.nbas, 16, 40, hl, ge, 10, 10, True, 1, esh)
        rel = np.abs(ge - se) / np.abs(se)
        worst = min(cos_sim(gb[i * 16:(i + 1) * 16], gc[i * 16:(i + 1) * 16], sb[i * 16:(i + 1) * 16],
                            sc[i * 16:(i + 1) * 16], hl.nbas) for i in range(40))
        rb, rc, re, _ = ref.intertwine(rb, rc, hl.nbas, 16, 40, hl, re, 10, 10, True, 1,
                                       IT.block_shift(re, bounds[1]))
        free = np.abs(ge - re) / np.abs(re)
        print(f"cycle {cyc + 1}: shadow eig {rel.max():.2e} vec {1 - worst:.2e}; free-running {free.max():.2e}")
        assert rel.max() <= CYCLE_EIG_RTOL, (cyc, rel.max())
        assert 1 - worst <= CYCLE_COS_TOL, (cyc, worst)


@pytest.mark.gpu
def test_solver_loop_from_product_guess(ref, cuda_device):
    """The first two cycles from the solver's product-function guess, whose
    augmentation terms carry weights of 1e-12 (AugmentVWithRandom's rule):
    the normal equations are then conditioned at the penalty's 1e10, and the
    double-word stages (about 48 bits) drift from the FP64 reference by a few
    1e-6 relative in the eigenvalues (measured 3.5e-6 at most over the 40
    states) before the fixed point pulls both together; bound 2e-5."""
    from mlcp_gb300 import hoplist as H
    from mlcp_gb300 import intertwine as IT
    from mlcp_gb300 import solver
    hl = H.henon_heiles(D=6, n=10, lam=0.111803)
    base, coef = solver.product_guess(hl.nbas, 40, 16)
    sb, sc = oracle.spectral_start(hl.nbas, 16)
    _, _, bounds = oracle.spectral_range(sb, sc, hl.nbas, 16, hl, 10, 5)
    e0 = oracle.qhq_diag(base, coef, hl.nbas, 16, 40, hl)
    gb, gc, ge = base.copy(), coef.copy(), e0.copy()
    rb, rc, re = base.copy(), coef.copy(), e0.copy()
    for cyc in range(2):
        gb, gc, ge = IT.intertwine(gb, gc, hl.nbas, 16, 40, hl, ge, 10, 10, True, 1, IT.block_shift(ge, bounds[1]))
        rb, rc, re, _ = ref.intertwine(rb, rc, hl.nbas, 16, 40, hl, re, 10, 10, True, 1,
                                       IT.block_shift(re, bounds[1]))
        rel = np.abs(ge - re) / np.abs(re)
        assert rel.max() <= 2e-5, (cyc, rel.max())
