"""GPU parity of the explicit-target ALS against the FP64 oracle.

The GPU contracts in FP32 (24-bit) and solves the normal equations in
double-word arithmetic (~48 bits).  Two checks per case:

* One sweep from a common state (the GPU's state after nals-1 sweeps): the
  relative residuals ||F - G|| / ||G|| of GPU and oracle agree to
  SWEEP_RES_TOL = 2e-7 (absolute difference) and the two results agree as
  functions, ||F_gpu - F_oracle|| / ||F_oracle|| <= SWEEP_VEC_TOL = 1e-5.
  This is the per-step precision of the FP32 contractions.
* The whole nals-sweep trajectory: residuals agree to TRAJ_RES_TOL = 5e-5
  and the vectors to TRAJ_VEC_TOL = 5e-4.  ALS trajectories of random
  low-rank fits converge slowly and carry perturbations forward: the FP64
  oracle itself, with nothing changed but its right-hand sides rounded to
  FP32 before each solve, moves by 1.7e-6 in residual and 6e-5 in distance
  after four sweeps on the 5-mode basis-16 case (pinned on the CPU in
  test_oracle.py::test_oracle_als_drift_under_fp32_rhs), and the GPU's
  FP32 sums over the target terms are noisier than one rounding.
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import als, workloads

SWEEP_RES_TOL = 2e-7
SWEEP_VEC_TOL = 1e-5
TRAJ_RES_TOL = 5e-5
TRAJ_VEC_TOL = 5e-4


def rel_residual(fc, fb, gc, gb, nbas):
    ff = oracle.cp_dot(fb, fc, fb, fc, nbas)
    gg = oracle.cp_dot(gb, gc, gb, gc, nbas)
    fg = oracle.cp_dot(fb, fc, gb, gc, nbas)
    return np.sqrt(max(ff + gg - 2 * fg, 0.0) / gg)


def rel_distance(ac, ab, bc, bb, nbas):
    aa = oracle.cp_dot(ab, ac, ab, ac, nbas)
    bbv = oracle.cp_dot(bb, bc, bb, bc, nbas)
    ab_ = oracle.cp_dot(ab, ac, bb, bc, nbas)
    return np.sqrt(max(aa + bbv - 2 * ab_, 0.0) / bbv)


def run_gpu(batch, nals, dev):
    import torch
    coef = torch.from_numpy(batch.coef.copy()).to(dev)
    base = torch.from_numpy(batch.base.copy()).to(dev)
    status = torch.zeros(batch.nvec, dtype=torch.int32, device=dev)
    als.reduce_batched(coef, base, batch.nbas, batch.rF, batch.rG, batch.term_off, nals, status=status)
    torch.cuda.synchronize()
    return coef.cpu().numpy(), base.cpu().numpy(), status.cpu().numpy()


CASES = [
    # (nvec, D, n, rF, rG, nals)
    (1, 4, [4, 5, 3, 6], 3, 12, 5),
    (3, 6, 12, [8, 5, 8], [64, 40, 17], 10),  # rank 17 is padded with zero weights for the oracle
    (2, 30, 12, 20, 200, 3),
    (4, 3, [9, 16, 7], 6, 30, 8),
    (40, 6, 10, 10, 2000, 3),  # 2-CTA clusters, 8 tiles per CTA: the staging ring wraps
    (2, 5, [20, 12, 40, 7, 17], 9, 150, 4),  # bases above 16: right-hand sides in several column rounds
    (1, 3, [6, 5, 4], 64, 256, 3),  # the largest F rank
    (2, 2, [10, 14], 5, 60, 6),  # two modes: the previous and the next mode coincide
]


def with_f_terms(batch, coef, base):
    """The batch with its F terms replaced by those of (coef, base)."""
    c, b = batch.coef.copy(), batch.base.copy()
    for v in range(batch.nvec):
        t0, f = int(batch.term_off[v]), int(batch.rF[v])
        c[t0:t0 + f] = coef[t0:t0 + f]
        b[t0:t0 + f] = base[t0:t0 + f]
    return workloads.AlsBatch(nbas=batch.nbas, rF=batch.rF, rG=batch.rG, term_off=batch.term_off, coef=c, base=b)


def compare(batch, gc_, gb_, nals, res_tol, vec_tol):
    for v in range(batch.nvec):
        c0, b0 = batch.vector(v)
        f = int(batch.rF[v])
        pc, pb, rGp = oracle.pad_target(c0, b0, f, int(batch.rG[v]))
        oc, ob = oracle.als(pc, pb, batch.nbas, f, rGp, nals)
        t0 = int(batch.term_off[v])
        fc, fb = gc_[t0:t0 + f], gb_[t0:t0 + f]
        gcoef, gbase = c0[f:], b0[f:]
        r_orc = rel_residual(oc, ob, gcoef, gbase, batch.nbas)
        r_gpu = rel_residual(fc, fb, gcoef, gbase, batch.nbas)
        dist = rel_distance(fc, fb, oc, ob, batch.nbas)
        assert abs(r_gpu - r_orc) <= res_tol, (v, r_gpu, r_orc)
        assert dist <= vec_tol, (v, dist)
        # target terms are untouched
        np.testing.assert_array_equal(gb_[t0 + f:t0 + f + int(batch.rG[v])], gbase)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_als_sweep_matches_oracle(case, cuda_device):
    nvec, D, n, rF, rG, nals = case
    batch = workloads.als_batch(nvec, D, n, rF, rG, seed=11 + nvec)
    if nals > 1:
        sc, sb, status = run_gpu(batch, nals - 1, cuda_device)
        assert not status.any()
        batch = with_f_terms(batch, sc, sb)
    gc_, gb_, status = run_gpu(batch, 1, cuda_device)
    assert not status.any()
    compare(batch, gc_, gb_, 1, SWEEP_RES_TOL, SWEEP_VEC_TOL)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES)
def test_als_trajectory_tracks_oracle(case, cuda_device):
    nvec, D, n, rF, rG, nals = case
    batch = workloads.als_batch(nvec, D, n, rF, rG, seed=11 + nvec)
    gc_, gb_, status = run_gpu(batch, nals, cuda_device)
    assert not status.any()
    compare(batch, gc_, gb_, nals, TRAJ_RES_TOL, TRAJ_VEC_TOL)


@pytest.mark.gpu
def test_alscpp_abi_matches_oracle(cuda_device):
    batch = workloads.als_batch(1, 5, [6, 8, 5, 7, 4], 4, 24, seed=5)
    c0, b0 = batch.vector(0)
    c, b = c0.copy(), b0.copy()
    als.alscpp(c, b, batch.nbas, 4, 24, 6)
    oc, ob = oracle.als(c0, b0, batch.nbas, 4, 24, 6)
    assert rel_distance(c[:4], b[:4], oc, ob, batch.nbas) <= TRAJ_VEC_TOL
    np.testing.assert_array_equal(b[4:], b0[4:])


@pytest.mark.gpu
def test_als_rejects_single_mode(cuda_device):
    batch = workloads.als_batch(1, 2, 5, 3, 9, seed=3)
    import torch
    coef = torch.from_numpy(batch.coef.copy()).to(cuda_device)
    base = torch.from_numpy(batch.base.copy()).to(cuda_device)
    with pytest.raises(Exception, match="ndof"):
        als.reduce_batched(coef, base, [10], batch.rF, batch.rG, batch.term_off, 2)


@pytest.mark.gpu
def test_als_zero_sweeps_leaves_data(cuda_device):
    batch = workloads.als_batch(2, 4, 5, 3, 9, seed=3)
    c, b, _ = run_gpu(batch, 0, cuda_device)
    np.testing.assert_array_equal(c, batch.coef)
    np.testing.assert_array_equal(b, batch.base)


@pytest.mark.gpu
def test_als_exact_target_converges(cuda_device):
    """A target that is exactly rank rF (terms duplicated) is reproduced."""
    rng = np.random.default_rng(0)
    nbas = np.array([4, 5, 3, 6], dtype=np.int32)
    nD = int(nbas.sum())
    rF = 3
    Ft = rng.normal(size=(rF, nD))
    ct = rng.uniform(0.5, 2, rF)
    base = np.vstack([rng.normal(size=(rF, nD)), Ft, Ft])
    coef = np.concatenate([np.ones(rF), 0.5 * ct, 0.5 * ct])
    batch = workloads.AlsBatch(nbas=nbas, rF=np.array([rF], np.int32), rG=np.array([2 * rF], np.int32),
                               term_off=np.array([0], np.int64), coef=coef, base=base)
    c, b, status = run_gpu(batch, 200, cuda_device)
    r = rel_residual(c[:rF], b[:rF], coef[rF:], base[rF:], nbas)
    assert r < 1e-5, r


@pytest.mark.gpu
def test_cp_dot_matches_oracle(cuda_device):
    import torch
    batch = workloads.als_batch(3, 5, [4, 6, 5, 3, 8], [3, 5, 2], [10, 7, 12], seed=9)
    coef = torch.from_numpy(batch.coef).to(cuda_device)
    base = torch.from_numpy(batch.base).to(cuda_device)
    out = torch.zeros(batch.nvec, dtype=torch.float64, device=cuda_device)
    xo = batch.term_off
    yo = batch.term_off + batch.rF
    als.cp_dot_batched(coef, base, batch.nbas, xo, batch.rF, yo, batch.rG, out)
    got = out.cpu().numpy()
    for v in range(batch.nvec):
        c0, b0 = batch.vector(v)
        f = int(batch.rF[v])
        ref = oracle.cp_dot(b0[:f], c0[:f], b0[f:], c0[f:], batch.nbas)
        assert abs(got[v] - ref) <= 1e-12 * max(1.0, abs(ref))


@pytest.mark.gpu
@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("case", [(6, 5, 8, 6, 90), (3, 4, [7, 5, 9, 6], [5, 8, 3], [40, 70, 25])])
def test_host_entry_matches_device_entry(case, pinned, cuda_device):
    """mlcp_als_batched_host (host buffers in and out) returns bit-for-bit
    what mlcp_als_batched returns on the same data, and writes back only the
    F terms: evenly spaced vectors with equal ranks take the strided copies,
    the ragged batch one copy per vector.  Pinned (mapped) arrays take the
    path whose conversion kernel reads the target terms from host memory;
    pageable ones are copied whole."""
    import torch
    nvec, D, n, rF, rG = case
    batch = workloads.als_batch(nvec, D, n, rF, rG, seed=17)
    dc, db, _ = run_gpu(batch, 3, cuda_device)
    if pinned:
        hc = torch.from_numpy(batch.coef.copy()).pin_memory().numpy()
        hb = torch.from_numpy(batch.base.copy()).pin_memory().numpy()
    else:
        hc, hb = batch.coef.copy(), batch.base.copy()
    als.reduce_batched_host(hc, hb, batch.nbas, batch.rF, batch.rG, batch.term_off, 3)
    np.testing.assert_array_equal(hc, dc)
    np.testing.assert_array_equal(hb, db)
    for v in range(batch.nvec):
        t0, f = int(batch.term_off[v]), int(batch.rF[v])
        np.testing.assert_array_equal(hb[t0 + f:t0 + f + int(batch.rG[v])], batch.base[t0 + f:t0 + f + int(batch.rG[v])])
