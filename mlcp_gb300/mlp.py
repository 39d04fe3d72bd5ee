"""Three-layer MLP of the learned ALS warm start, trained and run by the
library's own kernels (``csrc/mlp.cu``): tcgen05 BF16 GEMMs with FP32
accumulation, ReLU, mean-squared-error loss, Adam on FP32 master weights.

Shapes (every GEMM dimension padded as the kernels need): inputs
``in_dim`` -> ``hidden`` -> ``hidden`` -> ``out_dim``.  Rows (samples),
hidden and output widths are padded to multiples of 128 (they are the M of
some GEMM), the input width to a multiple of 64; padding rows and columns
are zero and masked out of the loss.

Data layout: BF16 activations row-major [rows][width]; each layer also keeps
the transposed copy [width][rows] that its weight-gradient GEMM reads, and
each weight matrix [out][in] its transposed BF16 copy [in][out] that the
input-gradient GEMM reads.  Torch allocates the device buffers; every
computation is a call into libmlcp_gb300.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _pad(x: int, m: int) -> int:
    return (x + m - 1) // m * m


def _ptr(t) -> int:
    return t.data_ptr()


def torch_stream():
    """Handle of torch's current stream for the library calls, so that they
    order with the torch operations that fill and read the buffers (the
    legacy default stream is passed as its special handle 1, since NULL
    selects the library's own stream)."""
    import torch
    return torch.cuda.current_stream().cuda_stream or 1


class Mlp:
    """MLP with device-resident parameters.  ``params()`` returns FP32 master
    copies (W1, b1, W2, b2, W3, b3) as numpy arrays of the logical shapes."""

    def __init__(self, in_dim: int, out_dim: int, hidden: int = 256, seed: int = 0, device=None):
        import torch
        self.torch = torch
        self.dev = device or torch.device("cuda", torch.cuda.current_device())
        self.in_dim, self.out_dim, self.hidden = in_dim, out_dim, hidden
        self.in_p = _pad(in_dim, 64)
        self.h_p = _pad(hidden, 128)
        self.out_p = _pad(out_dim, 128)
        rng = np.random.default_rng(seed)
        dims = [(self.h_p, self.in_p, hidden, in_dim), (self.h_p, self.h_p, hidden, hidden),
                (self.out_p, self.h_p, out_dim, hidden)]
        self.layers = []
        for (rp, cp, r, c) in dims:
            w = np.zeros((rp, cp), dtype=np.float32)
            w[:r, :c] = rng.uniform(-1.0, 1.0, size=(r, c)) * np.sqrt(3.0 / c)
            L = {"rows": rp, "cols": cp,
                 "w": torch.from_numpy(w).to(self.dev), "b": torch.zeros(rp, dtype=torch.float32, device=self.dev)}
            for k in ("mw", "vw"):
                L[k] = torch.zeros_like(L["w"])
            for k in ("mb", "vb"):
                L[k] = torch.zeros_like(L["b"])
            L["gw"] = torch.zeros_like(L["w"])
            L["gb"] = torch.zeros_like(L["b"])
            L["wb"] = L["w"].to(torch.bfloat16).contiguous()
            L["wt"] = L["w"].t().contiguous().to(torch.bfloat16)
            self.layers.append(L)
        self.step_no = 0
        self.status = torch.zeros(1, dtype=torch.int32, device=self.dev)
        self._rows = 0

    # -- buffers for a number of padded rows --
    def _buffers(self, rows_p: int):
        if rows_p == self._rows:
            return
        t = self.torch
        bf = t.bfloat16
        z = lambda r, c, dt=bf: t.zeros((r, c), dtype=dt, device=self.dev)  # noqa: E731
        self.H1, self.H1t = z(rows_p, self.h_p), z(self.h_p, rows_p)
        self.H2, self.H2t = z(rows_p, self.h_p), z(self.h_p, rows_p)
        self.Y = z(rows_p, self.out_p, t.float32)
        self.dY, self.dYt = z(rows_p, self.out_p), z(self.out_p, rows_p)
        self.dZ2, self.dZ2t = z(rows_p, self.h_p), z(self.h_p, rows_p)
        self.dZ1, self.dZ1t = z(rows_p, self.h_p), z(self.h_p, rows_p)
        self.Xt = z(self.in_p, rows_p)
        self.loss = t.zeros(1, dtype=t.float32, device=self.dev)
        self._rows = rows_p

    def _gemm(self, A, B, M, N, K, bias=None, act=0, mask=None, C=None, Cb=None, Ct=None, valid_m=None):
        L = _lib.load()
        rc = L.mlcp_mlp_gemm(_ptr(A), _ptr(B), M, N, K, A.shape[1], B.shape[1], _ptr(bias) if bias is not None else None,
                             act, _ptr(mask) if mask is not None else None, mask.shape[1] if mask is not None else 0,
                             _ptr(C) if C is not None else None, C.shape[1] if C is not None else 0,
                             _ptr(Cb) if Cb is not None else None, Cb.shape[1] if Cb is not None else 0,
                             _ptr(Ct) if Ct is not None else None, Ct.shape[1] if Ct is not None else 0,
                             M if valid_m is None else valid_m, _ptr(self.status), torch_stream())
        _lib.check(rc)

    def pad_inputs(self, X):
        """BF16 [rows_p][in_p] copy of X (rows x in_dim, any float dtype)."""
        t = self.torch
        rows = X.shape[0]
        rows_p = _pad(max(rows, 1), 128)
        Xp = t.zeros((rows_p, self.in_p), dtype=t.bfloat16, device=self.dev)
        Xp[:rows, :X.shape[1]] = X.to(t.bfloat16)
        return Xp, rows

    def forward(self, Xp, rows: int):
        """Xp: BF16 [rows_p][in_p] (pad_inputs).  Returns Y FP32 [rows_p][out_p]."""
        rows_p = Xp.shape[0]
        self._buffers(rows_p)
        L1, L2, L3 = self.layers
        self._gemm(Xp, L1["wb"], rows_p, self.h_p, self.in_p, bias=L1["b"], act=1, Cb=self.H1, Ct=self.H1t,
                   valid_m=rows)
        self._gemm(self.H1, L2["wb"], rows_p, self.h_p, self.h_p, bias=L2["b"], act=1, Cb=self.H2, Ct=self.H2t,
                   valid_m=rows)
        self._gemm(self.H2, L3["wb"], rows_p, self.out_p, self.h_p, bias=L3["b"], act=0, C=self.Y, valid_m=rows)
        return self.Y

    def backward(self, Xp, rows: int, T):
        """Gradients of the mean squared error of the last forward against T
        (FP32 [rows_p][out_p]; columns >= out_dim ignored) into each layer's
        gw/gb.  Returns the loss (device scalar)."""
        L = _lib.load()
        rows_p = Xp.shape[0]
        L1, L2, L3 = self.layers
        self.loss.zero_()
        _lib.check(L.mlcp_mlp_loss(_ptr(self.Y), _ptr(T), rows, self.out_dim, self.out_p, rows_p, _ptr(self.dY),
                                   _ptr(self.dYt), _ptr(self.loss), torch_stream()))
        self.Xt.copy_(Xp.t())
        # layer 3: dW3 = dY^T H2, db3 = colsum dY, dZ2 = (dY W3) * (H2 > 0)
        self._gemm(self.dYt, self.H2t, self.out_p, self.h_p, rows_p, C=L3["gw"])
        _lib.check(L.mlcp_mlp_colsum(_ptr(self.dY), rows_p, self.out_p, self.out_p, _ptr(L3["gb"]), torch_stream()))
        self._gemm(self.dY, L3["wt"], rows_p, self.h_p, self.out_p, act=2, mask=self.H2, Cb=self.dZ2, Ct=self.dZ2t,
                   valid_m=rows)
        # layer 2
        self._gemm(self.dZ2t, self.H1t, self.h_p, self.h_p, rows_p, C=L2["gw"])
        _lib.check(L.mlcp_mlp_colsum(_ptr(self.dZ2), rows_p, self.h_p, self.h_p, _ptr(L2["gb"]), torch_stream()))
        self._gemm(self.dZ2, L2["wt"], rows_p, self.h_p, self.h_p, act=2, mask=self.H1, Cb=self.dZ1, Ct=self.dZ1t,
                   valid_m=rows)
        # layer 1
        self._gemm(self.dZ1t, self.Xt, self.h_p, self.in_p, rows_p, C=L1["gw"])
        _lib.check(L.mlcp_mlp_colsum(_ptr(self.dZ1), rows_p, self.h_p, self.h_p, _ptr(L1["gb"]), torch_stream()))
        return self.loss

    def adam(self, lr: float = 1e-3, b1: float = 0.9, b2: float = 0.999, eps: float = 1e-8):
        L = _lib.load()
        self.step_no += 1
        for Ly in self.layers:
            _lib.check(L.mlcp_mlp_adam(_ptr(Ly["w"]), _ptr(Ly["gw"]), _ptr(Ly["mw"]), _ptr(Ly["vw"]), Ly["rows"],
                                       Ly["cols"], ctypes.c_float(lr), ctypes.c_float(b1), ctypes.c_float(b2),
                                       ctypes.c_float(eps), self.step_no, _ptr(Ly["wb"]), _ptr(Ly["wt"]), torch_stream()))
            _lib.check(L.mlcp_mlp_adam(_ptr(Ly["b"]), _ptr(Ly["gb"]), _ptr(Ly["mb"]), _ptr(Ly["vb"]), 1, Ly["rows"],
                                       ctypes.c_float(lr), ctypes.c_float(b1), ctypes.c_float(b2),
                                       ctypes.c_float(eps), self.step_no, None, None, torch_stream()))

    def check_status(self):
        if int(self.status.item()) != 0:
            raise _lib.MlcpError("mlp gemm: an internal wait timed out")

    def params(self):
        out = []
        for Ly, (r, c) in zip(self.layers, [(self.hidden, self.in_dim), (self.hidden, self.hidden),
                                            (self.out_dim, self.hidden)]):
            out.append(Ly["w"][:r, :c].cpu().numpy().astype(np.float64))
            out.append(Ly["b"][:r].cpu().numpy().astype(np.float64))
        return out

    def grads(self):
        out = []
        for Ly, (r, c) in zip(self.layers, [(self.hidden, self.in_dim), (self.hidden, self.hidden),
                                            (self.out_dim, self.hidden)]):
            out.append(Ly["gw"][:r, :c].cpu().numpy().astype(np.float64))
            out.append(Ly["gb"][:r].cpu().numpy().astype(np.float64))
        return out
