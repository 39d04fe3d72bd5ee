"""The warm-start MLP's kernels on the GPU (csrc/mlp.cu through the C ABI).

* The tcgen05 BF16 GEMM against an FP64 product of the same BF16 values:
  relative error of each entry at most 1e-5 of the row's largest |product|
  sum (FP32 accumulation over K), for several shapes (N not a multiple of the
  256-wide tile, two N tiles, K slices wrapping the two-stage ring), with bias,
  ReLU, the ReLU-derivative mask and the transposed BF16 output.
* Forward and backward of the three-layer MLP against the CPU oracle
  (oracle/mlp_oracle.py, BF16 roundings at the same points, FP64
  arithmetic): loss to 1e-4 relative, each gradient tensor to 1e-2 relative
  in the Frobenius norm (a BF16 rounding of an intermediate can flip by one
  unit, 2^-8, where FP32 and FP64 accumulation straddle a rounding boundary).
* Adam steps on a learnable map reduce the loss.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as MO


def bf(t):
    import torch
    return t.to(torch.bfloat16)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(128, 16, 64), (256, 144, 192), (384, 400, 128), (128, 256, 512)])
@pytest.mark.parametrize("act", [0, 1, 2])
def test_gemm_matches_fp64(shape, act, cuda_device):
    import torch
    from mlcp_gb300 import _lib
    from mlcp_gb300.mlp import torch_stream
    M, N, K = shape
    g = torch.Generator().manual_seed(M + N + K + act)
    A = bf(torch.randn(M, K, generator=g)).to(cuda_device)
    B = bf(torch.randn(N, K, generator=g)).to(cuda_device)
    bias = torch.randn(N, generator=g).float().to(cuda_device)
    mask = bf(torch.randn(M, N, generator=g)).to(cuda_device)
    C = torch.zeros(M, N, dtype=torch.float32, device=cuda_device)
    Cb = torch.zeros(M, N, dtype=torch.bfloat16, device=cuda_device)
    Ct = torch.zeros(N, M, dtype=torch.bfloat16, device=cuda_device)
    st = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    valid = M - 5
    L = _lib.load()
    rc = L.mlcp_mlp_gemm(A.data_ptr(), B.data_ptr(), M, N, K, K, K, bias.data_ptr(), act,
                         mask.data_ptr() if act == 2 else None, N, C.data_ptr(), N, Cb.data_ptr(), N, Ct.data_ptr(), M,
                         valid, st.data_ptr(), torch_stream())
    _lib.check(rc)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    a = A.float().cpu().double().numpy()
    b = B.float().cpu().double().numpy()
    ref = a @ b.T + bias.cpu().double().numpy()
    if act == 1:
        ref = np.maximum(ref, 0.0)
    if act == 2:
        ref = np.where(mask.float().cpu().numpy() > 0, ref, 0.0)
    ref[valid:] = 0.0
    scale = np.abs(a) @ np.abs(b).T + 1.0
    got = C.cpu().double().numpy()
    assert np.max(np.abs(got - ref) / scale) <= 1e-5
    gb = Cb.float().cpu().double().numpy()
    np.testing.assert_array_equal(gb, MO.bf16(got))
    np.testing.assert_array_equal(Ct.float().cpu().double().numpy(), gb.T)


def make_problem(seed=0, rows=300, din=576, dout=240):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(rows, din)) * 0.5
    Wt = rng.normal(size=(dout, din)) / np.sqrt(din)
    T = np.tanh(X @ Wt.T)
    return X, T


@pytest.mark.gpu
def test_mlp_gradients_match_oracle(cuda_device):
    import torch
    from mlcp_gb300.mlp import Mlp
    X, T = make_problem()
    net = Mlp(X.shape[1], T.shape[1], hidden=256, seed=3, device=cuda_device)
    Xp, rows = net.pad_inputs(torch.from_numpy(X).to(cuda_device))
    Tp = torch.zeros(Xp.shape[0], net.out_p, dtype=torch.float32, device=cuda_device)
    Tp[:rows, :T.shape[1]] = torch.from_numpy(T).float().to(cuda_device)
    net.forward(Xp, rows)
    loss = float(net.backward(Xp, rows, Tp).item())
    torch.cuda.synchronize()
    net.check_status()
    params = net.params()
    oloss, og = MO.loss_and_grads(params, X, T.astype(np.float32).astype(np.float64))
    assert abs(loss - oloss) <= 1e-4 * oloss, (loss, oloss)
    for k, (g, o) in enumerate(zip(net.grads(), og)):
        err = np.linalg.norm(g - o) / np.linalg.norm(o)
        assert err <= 1e-2, (k, err)


@pytest.mark.gpu
def test_mlp_training_reduces_loss(cuda_device):
    import torch
    from mlcp_gb300.mlp import Mlp
    X, T = make_problem(seed=4, rows=512)
    net = Mlp(X.shape[1], T.shape[1], hidden=256, seed=5, device=cuda_device)
    Xp, rows = net.pad_inputs(torch.from_numpy(X).to(cuda_device))
    Tp = torch.zeros(Xp.shape[0], net.out_p, dtype=torch.float32, device=cuda_device)
    Tp[:rows, :T.shape[1]] = torch.from_numpy(T).float().to(cuda_device)
    losses = []
    for _ in range(200):
        net.forward(Xp, rows)
        losses.append(float(net.backward(Xp, rows, Tp).item()))
        net.adam(lr=1e-3)
    net.check_status()
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
