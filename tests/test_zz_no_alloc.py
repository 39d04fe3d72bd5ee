"""The allocation-free ALS entry point (mlcp_als_noalloc) against the
allocating one (mlcp_als_batched), through the C ABI.

Some callers cannot allocate device memory when they reduce a vector: hosts
whose device memory is owned up front by another allocator or memory pool,
and latency-critical loops that must stay out of the CUDA allocator.
mlcp_als_noalloc serves them from a fixed scratch array inside the library.

Checks: two calls in a row on different inputs match the allocating entry
point within the ALS test tolerances (relative residuals to 1e-6, reduced
vectors to 1e-4 as functions) and report a clear status word; the second call
does not change the device's free memory; a size beyond the fixed scratch is
rejected with a message, and so is a call without a status word (also with
nals = 0).
This file is collected last so that a run stopping at its first failure has
run every other test before it.
"""
import ctypes

import numpy as np
import pytest

import oracle
from mlcp_gb300 import _lib, als, workloads

RES_TOL = 1e-6
VEC_TOL = 1e-4

_I = ctypes.POINTER(ctypes.c_int)


def _noalloc(coef, base, nbas, rF, rG, nals, stream, status):
    nb = np.ascontiguousarray(nbas, dtype=np.int32)
    L = _lib.load()
    rc = L.mlcp_als_noalloc(len(nb), nb.ctypes.data_as(_I), int(rF), int(rG), coef.data_ptr(), base.data_ptr(),
                            int(nals), None if status is None else status.data_ptr(), stream)
    return rc


def _rel(ac, ab, bc, bb, nbas):
    aa = oracle.cp_dot(ab, ac, ab, ac, nbas)
    bbv = oracle.cp_dot(bb, bc, bb, bc, nbas)
    x = oracle.cp_dot(ab, ac, bb, bc, nbas)
    return np.sqrt(max(aa + bbv - 2 * x, 0.0) / bbv)


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point(cuda_device):
    import torch
    stream = torch.cuda.current_stream(cuda_device)
    handle = stream.cuda_stream if stream.cuda_stream != 0 else 1
    free_after_first = None
    for call, seed in enumerate((101, 202)):
        batch = workloads.als_batch(1, 6, [8, 12, 5, 9, 12, 7], 6, 48, seed=seed)
        c0, b0 = batch.vector(0)
        # existing (allocating) entry point
        ca = torch.from_numpy(c0.copy()).to(cuda_device)
        ba = torch.from_numpy(b0.copy()).to(cuda_device)
        als.reduce_batched(ca, ba, batch.nbas, [6], [48], [0], 5)
        # allocation-free entry point on its own copy
        cn = torch.from_numpy(c0.copy()).to(cuda_device)
        bn = torch.from_numpy(b0.copy()).to(cuda_device)
        torch.cuda.synchronize()
        st = torch.full((1,), -1, dtype=torch.int32, device=cuda_device)
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info(cuda_device)[0]
        rc = _noalloc(cn, bn, batch.nbas, 6, 48, 5, handle, st)
        assert rc == 0, _lib.last_error()
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info(cuda_device)[0] == free_before
        assert int(st.item()) == 0
        fa, fba = ca.cpu().numpy()[:6], ba.cpu().numpy()[:6]
        fn, fbn = cn.cpu().numpy()[:6], bn.cpu().numpy()[:6]
        g_c, g_b = c0[6:], b0[6:]
        ra, rn = _rel(fa, fba, g_c, g_b, batch.nbas), _rel(fn, fbn, g_c, g_b, batch.nbas)
        assert abs(ra - rn) <= RES_TOL, (call, ra, rn)
        assert _rel(fn, fbn, fa, fba, batch.nbas) <= VEC_TOL
        np.testing.assert_array_equal(bn.cpu().numpy()[6:], b0[6:])


@pytest.mark.gpu
def test_noalloc_rejects_oversized_target(cuda_device):
    import torch
    # fits the shared-memory plan, but its FP32 target copy alone (30000 terms
    # x 360 basis functions) exceeds the fixed scratch array
    nbas = np.full(30, 12, dtype=np.int32)
    coef = torch.zeros(20 + 30000, dtype=torch.float64, device=cuda_device)
    base = torch.zeros((20 + 30000) * int(nbas.sum()), dtype=torch.float64, device=cuda_device)
    st = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    rc = _noalloc(coef, base, nbas, 20, 30000, 1, None, st)
    assert rc != 0
    assert "scratch" in _lib.last_error()


@pytest.mark.gpu
def test_noalloc_requires_status_word(cuda_device):
    """Without d_status a timed-out wait or a singular solve could not be
    reported, so the call is refused before any work, also with nals = 0."""
    import torch
    batch = workloads.als_batch(1, 4, 5, 3, 9, seed=3)
    c0, b0 = batch.vector(0)
    coef = torch.from_numpy(c0.copy()).to(cuda_device)
    base = torch.from_numpy(b0.copy()).to(cuda_device)
    for nals in (0, 2):
        rc = _noalloc(coef, base, batch.nbas, 3, 9, nals, None, None)
        assert rc != 0
        assert "d_status" in _lib.last_error()
    np.testing.assert_array_equal(base.cpu().numpy(), b0)
