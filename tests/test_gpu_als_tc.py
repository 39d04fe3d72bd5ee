"""The tensor-core form of the batched ALS (engine 2: per-mode dot products
as tcgen05 MMAs on BF16 three-way splits with FP32 accumulation, running
products in tensor memory) against the FP64 oracle, with the tolerances of
the CUDA-core form (tests/test_gpu_als.py): one sweep from a common state
to SWEEP_RES_TOL = 2e-7 in residual and 1e-5 as functions; whole
trajectories to 5e-5 and 5e-4.  The split keeps every dot product to about
2^-26 of its terms (the dropped piece products), below the FP32 rounding
of the CUDA-core dots, so the same bounds apply.

Each case checks, through the autotuner's report, that the tensor-core form
is the one that ran wherever one of its launch shapes fits.  The benchmark's
shape (30 modes of 12, 3200 -> 20 terms, 10 sweeps) is checked on eight of
its vectors against the oracle's residuals (1e-6 relative), and against the
CUDA-core form of the same batch.
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import _lib, workloads

from test_gpu_als import (CASES, SWEEP_RES_TOL, SWEEP_VEC_TOL, TRAJ_RES_TOL, TRAJ_VEC_TOL, compare, rel_residual,
                          run_gpu, with_f_terms)


@pytest.fixture
def tensor_engine(cuda_device):
    _lib.set_als_engine(2)
    yield cuda_device
    _lib.set_als_engine(0)


def ran_tensor_form(batch) -> bool:
    """The autotuner's entry for this shape under engine 2 chose the
    tensor-core form, or, when no tensor-core candidate fits the shared
    memory (bases above 16 need wide operand buffers besides a ring of at
    least three stages), it tried none and fell back to the CUDA-core form."""
    nD = int(np.sum(batch.nbas))
    key = f"als nvec={batch.nvec} ndof={len(batch.nbas)} nD={nD} "
    lines = [ln for ln in _lib.autotune_report().splitlines() if ln.startswith(key) and "engine=2" in ln]
    if not lines:
        return False
    for ln in lines:
        head, _, trials = ln.partition(";")
        tried_tc = any(t.split("=")[0].endswith("t") for t in trials.split())
        if head.endswith(" tensor") != tried_tc:
            return False
    return True


TC_CASES = [c for c in CASES if max(np.atleast_1d(c[3])) <= 32]


@pytest.mark.gpu
@pytest.mark.parametrize("case", TC_CASES)
def test_tensor_form_sweep_matches_oracle(case, tensor_engine):
    nvec, D, n, rF, rG, nals = case
    batch = workloads.als_batch(nvec, D, n, rF, rG, seed=11 + nvec)
    if nals > 1:
        sc, sb, status = run_gpu(batch, nals - 1, tensor_engine)
        assert not status.any()
        batch = with_f_terms(batch, sc, sb)
    gc_, gb_, status = run_gpu(batch, 1, tensor_engine)
    assert not status.any()
    assert ran_tensor_form(batch), _lib.autotune_report()
    compare(batch, gc_, gb_, 1, SWEEP_RES_TOL, SWEEP_VEC_TOL)


@pytest.mark.gpu
@pytest.mark.parametrize("case", TC_CASES)
def test_tensor_form_trajectory_tracks_oracle(case, tensor_engine):
    nvec, D, n, rF, rG, nals = case
    batch = workloads.als_batch(nvec, D, n, rF, rG, seed=11 + nvec)
    gc_, gb_, status = run_gpu(batch, nals, tensor_engine)
    assert not status.any()
    compare(batch, gc_, gb_, nals, TRAJ_RES_TOL, TRAJ_VEC_TOL)


@pytest.mark.gpu
def test_tensor_form_benchmark_shape(tensor_engine):
    batch = workloads.als_batch(8, 30, 12, 20, 3200, seed=workloads.ALS_SEED)
    tc_c, tc_b, status = run_gpu(batch, 10, tensor_engine)
    assert not status.any()
    assert ran_tensor_form(batch), _lib.autotune_report()
    _lib.set_als_engine(1)
    cc_c, cc_b, status = run_gpu(batch, 10, tensor_engine)
    assert not status.any()
    coefs, bases = [], []
    for v in range(batch.nvec):
        c0, b0 = batch.vector(v)
        coefs.append(np.ascontiguousarray(c0))
        bases.append(np.ascontiguousarray(b0))
    oracle.als_batched(coefs, bases, batch.nbas, list(batch.rF), list(batch.rG), 10)
    for v in range(batch.nvec):
        c0, b0 = batch.vector(v)
        t0 = int(batch.term_off[v])
        g = (c0[20:], b0[20:])
        r_orc = rel_residual(coefs[v][:20], bases[v][:20], *g, batch.nbas)
        r_tc = rel_residual(tc_c[t0:t0 + 20], tc_b[t0:t0 + 20], *g, batch.nbas)
        r_cc = rel_residual(cc_c[t0:t0 + 20], cc_b[t0:t0 + 20], *g, batch.nbas)
        assert abs(r_tc - r_orc) <= 1e-6 * r_orc, (v, r_tc, r_orc)
        assert abs(r_cc - r_orc) <= 1e-6 * r_orc, (v, r_cc, r_orc)
