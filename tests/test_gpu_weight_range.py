"""Exponent range of the in-place power sweep (POW_ALS, reference
src/intertw_mvp.cu:452-497, sweep loop :468-494).

The reference applies (H - E) once per mode step and renormalises the CP
weights only at the end of a sweep, so within a sweep the weights grow by
about ||H - E|| per step.  In FP64 that is harmless; the GPU sweep carries
the weights and right-hand sides in double-word arithmetic (FP32 exponent
range), so it rescales the weights by a power of two after every step (the
end-of-sweep renormalisation removes any common factor).

Check: the same power cycle on H and on 2^40 H (shift scaled alike).  A
power-of-two scale changes no rounding, so the two results agree to the last
few bits (1e-10 here), and the scaled run agrees with the FP64 oracle to the
cycle tests' tolerance.  Without the rescale the scaled run's weights reach
about 1e13 after one step and its squared row norms overflow FP32 in the
second, which the cycle reports as a non-positive-definite matrix.
"""
import numpy as np
import pytest

import oracle
from mlcp_gb300 import hoplist as H
from mlcp_gb300 import intertwine as IT

SCALE = 2.0 ** 40

CASES = [
    # (hoplist factory, rk, nbloc, npow, ishift, Eshift)
    (lambda: H.henon_heiles(D=4, n=6), 6, 5, 3, 1, 6.0),
    (lambda: H.random_hoplist([6, 4, 5, 3], 9, seed=8, coupling=3), 4, 3, 2, -1, 1.5),
]


def scaled(hl, s):
    return H.HopList(nbas=hl.nbas, opid=hl.opid, mptr=hl.mptr, coef=hl.coef * s, mat=hl.mat)


def cos_sim(ab, ac, bb, bc, nbas):
    aa = oracle.cp_dot(ab, ac, ab, ac, nbas)
    bbv = oracle.cp_dot(bb, bc, bb, bc, nbas)
    return abs(oracle.cp_dot(ab, ac, bb, bc, nbas)) / np.sqrt(aa * bbv)


@pytest.mark.gpu
@pytest.mark.parametrize("case", range(len(CASES)))
def test_power_sweep_is_scale_free(case, cuda_device):
    make, rk, nbloc, npow, ishift, esh = CASES[case]
    hl = make()
    big = scaled(hl, SCALE)
    rng = np.random.default_rng(50 + case)
    Q = rng.uniform(-0.5, 0.5, size=(rk * nbloc, int(np.sum(hl.nbas))))
    qc = np.ones(rk * nbloc)
    eig0 = np.zeros(nbloc)
    ab, ac, _ = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, hl, eig0, npow, 0, False, ishift, esh)
    bb, bc, _ = IT.intertwine(Q, qc, hl.nbas, rk, nbloc, big, eig0, npow, 0, False, ishift, esh * SCALE)
    ob, oc, _ = oracle.intertwine(Q, qc, hl.nbas, rk, nbloc, big, eig0, npow, 0, False, ishift, esh * SCALE)
    assert np.isfinite(bc).all() and np.isfinite(bb).all()
    np.testing.assert_allclose(bc, ac, rtol=1e-10, atol=1e-12)
    for i in range(nbloc):
        s = slice(i * rk, (i + 1) * rk)
        assert 1 - cos_sim(bb[s], bc[s], ab[s], ac[s], hl.nbas) <= 1e-10
        assert 1 - cos_sim(bb[s], bc[s], ob[s], oc[s], hl.nbas) <= 1e-6
