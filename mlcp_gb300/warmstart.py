"""Learned warm start of the explicit-target ALS reduction.

The reference starts its GPU ALS (alscpp_, called by GPU_ALS_AA,
src/GPUIterate.f90:191-210) from a random CP vector (GetRandomCPvec,
src/SepdRepn.f90:340-358: entries uniform in [-0.5, 0.5), weights 1).  Here a
three-layer MLP (width 256, BF16 weights, FP32 accumulation; ``mlp.py``)
proposes the starting factors instead, from the unreduced vector itself:

* features, per (vector, mode): the mode's factors of the vector's 64
  largest-weight target terms (unit, largest entry positive) and their
  log-weights (``mlcp_ws_features``);
* output: the mode's factors of the rank-R reduction (``mlcp_ws_apply``),
  one slot per input term among the R largest, one network shared by all
  modes of the same basis size;
* training pairs: (unreduced vector, converged reduction) from reductions
  the solver has already run (``collect``: ``mlcp_ws_targets`` matches each
  slot's input term with the reduction term it turned into);
* the acceptance test: both starts run the same fixed number of sweeps, and the
  proposal is accepted, vector by vector, when its relative residual
  ||F - G|| / ||G|| is no larger than the random start's; otherwise the
  random start's result is kept (the fallback).

``WarmStart.reduce`` returns, besides the reduced batch, the accept rate
and the sweeps saved: for each accepted vector, how many more sweeps the
random start needs to reach the accepted residual.
"""
from __future__ import annotations

import numpy as np

from . import _lib, als, workloads
from .mlp import Mlp, torch_stream

NTOP = 64


class WarmStart:
    """MLP warm start for reductions of rank ``rank`` over ``ndof`` modes of
    ``n`` basis functions each."""

    def __init__(self, ndof: int, n: int, rank: int, hidden: int = 256, seed: int = 0, device=None):
        import torch
        self.torch = torch
        self.dev = device or torch.device("cuda", torch.cuda.current_device())
        self.ndof, self.n, self.rank = ndof, n, rank
        self.in_dim = NTOP * (n + 1)
        self.out_dim = rank * n
        self.net = Mlp(self.in_dim, self.out_dim, hidden=hidden, seed=seed, device=self.dev)
        self.X = []   # feature rows (BF16, device)
        self.T = []   # targets (FP32, device)
        self.trained_on = 0

    # -- device views of a batch --
    def _meta(self, batch: workloads.AlsBatch):
        t = self.torch
        g_off = t.as_tensor(batch.term_off + batch.rF, dtype=t.int64, device=self.dev)
        g_rank = t.as_tensor(batch.rG, dtype=t.int32, device=self.dev)
        f_off = t.as_tensor(batch.term_off, dtype=t.int64, device=self.dev)
        return g_off, g_rank, f_off, int(batch.rG.max())

    def features(self, batch, coef, base):
        """BF16 feature rows [nvec*ndof][in_dim] of the batch's targets."""
        t = self.torch
        g_off, g_rank, _, rgmax = self._meta(batch)
        X = t.zeros((batch.nvec * self.ndof, self.in_dim), dtype=t.bfloat16, device=self.dev)
        L = _lib.load()
        _lib.check(L.mlcp_ws_features(batch.nvec, self.ndof, self.n, NTOP, g_off.data_ptr(), g_rank.data_ptr(), rgmax,
                                      base.data_ptr(), coef.data_ptr(), X.data_ptr(), self.in_dim, torch_stream()))
        return X

    def collect(self, batch, coef, base):
        """Add the pairs of a batch whose F terms hold converged reductions of
        its targets (the device arrays after a full reduction)."""
        t = self.torch
        X = self.features(batch, coef, base)
        g_off, g_rank, f_off, rgmax = self._meta(batch)
        T = t.zeros((batch.nvec * self.ndof, self.out_dim), dtype=t.float32, device=self.dev)
        L = _lib.load()
        _lib.check(L.mlcp_ws_targets(batch.nvec, self.ndof, self.n, self.rank, g_off.data_ptr(), g_rank.data_ptr(),
                                     rgmax, f_off.data_ptr(), base.data_ptr(), coef.data_ptr(), T.data_ptr(),
                                     self.out_dim, torch_stream()))
        self.X.append(X)
        self.T.append(T)

    def train(self, epochs: int = 300, lr: float = 1e-3):
        """Full-batch Adam on every pair collected so far; returns the losses."""
        t = self.torch
        X = t.cat(self.X)
        T = t.cat(self.T)
        Xp, rows = self.net.pad_inputs(X)
        Tp = t.zeros((Xp.shape[0], self.net.out_p), dtype=t.float32, device=self.dev)
        Tp[:rows, :self.out_dim] = T
        losses = []
        for _ in range(epochs):
            self.net.forward(Xp, rows)
            losses.append(self.net.backward(Xp, rows, Tp).clone())
            self.net.adam(lr=lr)
        self.net.check_status()
        self.trained_on = rows
        return [float(x.item()) for x in losses]

    def propose(self, batch, coef, base):
        """Overwrite the F terms of the device batch with the MLP's proposal."""
        X = self.features(batch, coef, base)
        Xp, rows = self.net.pad_inputs(X)
        Y = self.net.forward(Xp, rows)
        g_off, g_rank, f_off, rgmax = self._meta(batch)
        L = _lib.load()
        _lib.check(L.mlcp_ws_apply(batch.nvec, self.ndof, self.n, self.rank, g_off.data_ptr(), g_rank.data_ptr(),
                                   rgmax, f_off.data_ptr(), base.data_ptr(), coef.data_ptr(), Y.data_ptr(),
                                   self.net.out_p, torch_stream()))
        self.net.check_status()

    # -- the reduction with the acceptance test --
    def reduce(self, batch, fixed_sweeps: int, max_sweeps: int, seed: int = 0):
        """Reduce a device copy of the batch from the proposal and from the
        random start for fixed_sweeps each; keep, per vector, the better
        (accept the proposal when its residual is not larger).  Returns
        (coef, base, stats) with stats: accept_rate, sweeps_saved (mean over
        accepted vectors; the random start's residual history is followed up to
        max_sweeps), and both residual arrays."""
        t = self.torch
        random_batch = random_start(batch, seed)
        c_r = t.from_numpy(random_batch.coef).to(self.dev)
        b_r = t.from_numpy(random_batch.base).to(self.dev)
        c_m = c_r.clone()
        b_m = b_r.clone()
        self.propose(batch, c_m, b_m)
        st = t.zeros(batch.nvec, dtype=t.int32, device=self.dev)
        als.reduce_batched(c_m, b_m, batch.nbas, batch.rF, batch.rG, batch.term_off, fixed_sweeps, status=st,
                           stream=t.cuda.current_stream(self.dev))
        r_mlp = residuals(batch, c_m, b_m)
        # the random start, one sweep at a time, its residual after each
        hist = []
        for s in range(max_sweeps):
            als.reduce_batched(c_r, b_r, batch.nbas, batch.rF, batch.rG, batch.term_off, 1, status=st,
                               stream=t.cuda.current_stream(self.dev))
            hist.append(residuals(batch, c_r, b_r))
            if s + 1 == fixed_sweeps:
                c_fix, b_fix = c_r.clone(), b_r.clone()
        hist = np.array(hist)  # [sweeps][nvec]
        r_plain = hist[fixed_sweeps - 1]
        accept = r_mlp <= r_plain
        saved = []
        for v in np.nonzero(accept)[0]:
            reach = np.nonzero(hist[:, v] <= r_mlp[v])[0]
            need = (reach[0] + 1) if reach.size else max_sweeps
            saved.append(need - fixed_sweeps)
        # per vector: the accepted proposal's terms, else the random start's
        out_c, out_b = c_m.clone(), b_m.clone()
        for v in np.nonzero(~accept)[0]:
            t0, f = int(batch.term_off[v]), int(batch.rF[v])
            out_c[t0:t0 + f] = c_fix[t0:t0 + f]
            out_b[t0:t0 + f] = b_fix[t0:t0 + f]
        stats = {"accept_rate": float(accept.mean()), "sweeps_saved": float(np.mean(saved)) if saved else 0.0,
                 "fixed_sweeps": fixed_sweeps, "residual_mlp": r_mlp, "residual_random": r_plain,
                 "random_history": hist}
        return out_c, out_b, stats


def random_start(batch: workloads.AlsBatch, seed: int) -> workloads.AlsBatch:
    """The batch with every F replaced by GetRandomCPvec's start: factor
    entries uniform in [-0.5, 0.5), weights 1 (src/SepdRepn.f90:340-358)."""
    rng = np.random.default_rng(seed)
    c, b = batch.coef.copy(), batch.base.copy()
    for v in range(batch.nvec):
        t0, f = int(batch.term_off[v]), int(batch.rF[v])
        b[t0:t0 + f] = rng.uniform(-0.5, 0.5, size=(f, batch.nD))
        c[t0:t0 + f] = 1.0
    return workloads.AlsBatch(nbas=batch.nbas, rF=batch.rF, rG=batch.rG, term_off=batch.term_off, coef=c, base=b)


def residuals(batch, coef, base) -> np.ndarray:
    """||F - G|| / ||G|| per vector of a device batch (FP64, on the GPU)."""
    import torch
    dev = coef.device
    xo = batch.term_off
    yo = batch.term_off + batch.rF
    out = torch.zeros((3, batch.nvec), dtype=torch.float64, device=dev)
    als.cp_dot_batched(coef, base, batch.nbas, xo, batch.rF, xo, batch.rF, out[0])
    als.cp_dot_batched(coef, base, batch.nbas, yo, batch.rG, yo, batch.rG, out[1])
    als.cp_dot_batched(coef, base, batch.nbas, xo, batch.rF, yo, batch.rG, out[2])
    ff, gg, fg = out.cpu().numpy()
    return np.sqrt(np.maximum(ff + gg - 2 * fg, 0.0) / gg)


def power_steps(ws: WarmStart, hl, nvec: int, shift: float, ncycle: int = 8, train_cycles: int = 5,
                train_sweeps: int = 20, epochs: int = 600, fixed_sweeps: int = 3, max_sweeps: int = 20, seed: int = 0,
                device=None):
    """The warm start inside a power iteration: each cycle reduces
    (H - shift) F_v / ||.|| back to rank ws.rank for nvec vectors (the
    unreduced vectors of power steps, workloads.power_batch).  Cycles
    1..train_cycles are the solver's own reductions -- each started from the
    vector's previous iterate (a random start in cycle 1), train_sweeps sweeps
    -- and their pairs train the MLP; later cycles are tested reductions
    (WarmStart.reduce) whose result feeds the next cycle.  Returns
    (training losses, per tested cycle stats, seconds spent training)."""
    import time

    import torch

    from . import hoplist as H  # noqa: F401
    dev = device or ws.dev
    rank = ws.rank
    nD = int(np.sum(hl.nbas))
    rng = np.random.default_rng(seed)
    F = [(rng.uniform(-0.5, 0.5, size=(rank, nD)), np.ones(rank)) for _ in range(nvec)]
    losses, stats, t_train = None, [], 0.0
    for c in range(ncycle):
        batch = workloads.power_batch(hl, [f[0] for f in F], [f[1] for f in F], rank, shift=shift)
        if c < train_cycles:
            if c == 0:
                start = random_start(batch, seed=100)
            else:
                cb, bb = batch.coef.copy(), batch.base.copy()
                for v in range(nvec):
                    t0 = int(batch.term_off[v])
                    bb[t0:t0 + rank] = F[v][0]
                    cb[t0:t0 + rank] = F[v][1]
                start = workloads.AlsBatch(nbas=batch.nbas, rF=batch.rF, rG=batch.rG, term_off=batch.term_off,
                                           coef=cb, base=bb)
            coef = torch.from_numpy(start.coef).to(dev)
            base = torch.from_numpy(start.base).to(dev)
            st = torch.zeros(nvec, dtype=torch.int32, device=dev)
            als.reduce_batched(coef, base, batch.nbas, batch.rF, batch.rG, batch.term_off, train_sweeps, status=st)
            if bool(st.any()):
                raise _lib.MlcpError("warm start: a training reduction reported a non-positive pivot")
            ws.collect(batch, coef, base)
            if c == train_cycles - 1:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                losses = ws.train(epochs=epochs)
                t_train = time.perf_counter() - t0
        else:
            coef, base, s = ws.reduce(batch, fixed_sweeps=fixed_sweeps, max_sweeps=max_sweeps, seed=100 + c)
            s["cycle"] = c + 1
            stats.append(s)
        cn, bn = coef.cpu().numpy(), base.cpu().numpy()
        F = [(bn[int(batch.term_off[v]):int(batch.term_off[v]) + rank].copy(),
              cn[int(batch.term_off[v]):int(batch.term_off[v]) + rank].copy()) for v in range(nvec)]
    return losses, stats, t_train
