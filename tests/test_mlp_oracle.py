"""The warm-start MLP's CPU oracle (oracle/mlp_oracle.py) pinned on the CPU:
its FP64 gradients against central finite differences, and its BF16
rounding against known values."""
import numpy as np

from oracle import mlp_oracle as M


def small_net(seed=0, din=12, h=10, dout=7):
    rng = np.random.default_rng(seed)
    params = [rng.normal(size=(h, din)) / np.sqrt(din), rng.normal(size=h) * 0.1,
              rng.normal(size=(h, h)) / np.sqrt(h), rng.normal(size=h) * 0.1,
              rng.normal(size=(dout, h)) / np.sqrt(h), rng.normal(size=dout) * 0.1]
    X = rng.normal(size=(9, din))
    T = rng.normal(size=(9, dout))
    return params, X, T


def test_fp64_gradients_match_finite_differences():
    params, X, T = small_net()
    _, g = M.loss_and_grads(params, X, T, bf16_points=False)
    rng = np.random.default_rng(1)
    for which, p in enumerate(params):
        for _ in range(6):
            idx = tuple(int(rng.integers(0, s)) for s in p.shape)
            fd = M.finite_difference(params, X, T, which, idx)
            assert abs(fd - g[which][idx]) <= 1e-7 * max(1.0, abs(fd)), (which, idx, fd, g[which][idx])


def test_bf16_rounding():
    # 1 + 2^-8 is halfway between 1 and 1 + 2^-7: ties to even -> 1
    assert M.bf16(1.0 + 2.0 ** -8) == 1.0
    assert M.bf16(1.0 + 3 * 2.0 ** -8) == 1.0 + 2.0 ** -6
    assert M.bf16(-3.140625) == -3.140625
    x = np.random.default_rng(2).normal(size=1000)
    r = M.bf16(x)
    assert np.max(np.abs(r - x) / np.abs(x)) <= 2.0 ** -8
