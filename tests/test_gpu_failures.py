"""Failure detection without a GPU fault: each failure is reported as a
status or an error return, and the CUDA context stays usable afterwards.

* A pipeline wait that runs out: mlcp_gb300_wait_selftest waits, with the
  ALS kernel's own bounded tile wait, for a tile that is never issued; the
  wait gives up and reports the status bit the ALS kernel uses (2), and the
  next reduction is clean and bit-identical to one before.
* Non-finite normal equations (a NaN in one vector's starting factor of a
  mode that enters the first step's equations): that vector reports bit 0,
  the others are unaffected.
* An allocation the device cannot satisfy: an error return naming
  cudaMalloc, after which calls succeed again.
"""
import numpy as np
import pytest

from mlcp_gb300 import _lib, als, workloads


def run(batch, nals, dev, coef=None):
    import torch
    c = torch.from_numpy((batch.coef if coef is None else coef).copy()).to(dev)
    b = torch.from_numpy(batch.base.copy()).to(dev)
    st = torch.zeros(batch.nvec, dtype=torch.int32, device=dev)
    als.reduce_batched(c, b, batch.nbas, batch.rF, batch.rG, batch.term_off, nals, status=st)
    torch.cuda.synchronize()
    return c.cpu().numpy(), b.cpu().numpy(), st.cpu().numpy()


@pytest.mark.gpu
def test_pipeline_wait_timeout_is_reported(cuda_device):
    import ctypes
    import time
    batch = workloads.als_batch(3, 4, 6, 4, 600, seed=41)
    c0, b0, s0 = run(batch, 2, cuda_device)
    assert not s0.any()
    L = _lib.load()
    flags = ctypes.c_int(-1)
    t0 = time.perf_counter()
    assert L.mlcp_gb300_wait_selftest(ctypes.byref(flags)) == 0, _lib.last_error()
    assert time.perf_counter() - t0 < 30.0
    assert flags.value == 2
    c2, b2, s2 = run(batch, 2, cuda_device)
    assert not s2.any()
    np.testing.assert_array_equal(c2, c0)
    np.testing.assert_array_equal(b2, b0)


@pytest.mark.gpu
def test_nan_factor_flags_only_its_vector(cuda_device):
    batch = workloads.als_batch(3, 3, 5, 4, 128, seed=42)
    c0, b0, _ = run(batch, 2, cuda_device)
    bad = batch.base.copy()
    # mode 1 of the first F term: mode 0 is solved first and would simply be
    # replaced, but mode 1 enters the first step's normal equations
    bad[int(batch.term_off[1]), int(batch.nbas[0])] = np.nan
    poisoned = workloads.AlsBatch(nbas=batch.nbas, rF=batch.rF, rG=batch.rG, term_off=batch.term_off,
                                  coef=batch.coef, base=bad)
    c1, b1, s1 = run(poisoned, 2, cuda_device)
    assert int(s1[1]) & 1, s1
    assert s1[0] == 0 and s1[2] == 0, s1
    for v in (0, 2):
        t0 = int(batch.term_off[v])
        sl = slice(t0, t0 + int(batch.rF[v]))
        np.testing.assert_array_equal(c1[sl], c0[sl])
        np.testing.assert_array_equal(b1[sl], b0[sl])


@pytest.mark.gpu
def test_allocation_failure_is_an_error_return(cuda_device):
    """A batch whose device copy would need about 1.1 TB: the host-buffer
    entry returns an error before touching the (small) host arrays."""
    nbas = [64, 64]
    rG = 1 << 30
    coef = np.ones(8)
    base = np.ones((8, 128))
    with pytest.raises(_lib.MlcpError, match="cudaMalloc"):
        als.reduce_batched_host(coef, base, nbas, [4], [rG], [0], 2)
    batch = workloads.als_batch(2, 3, 5, 3, 60, seed=43)
    hc, hb = batch.coef.copy(), batch.base.copy()
    als.reduce_batched_host(hc, hb, batch.nbas, batch.rF, batch.rG, batch.term_off, 2)
    assert np.isfinite(hc).all()
