"""The learned ALS warm start (mlcp_gb300/warmstart.py) on power-step
reductions of a synthetic quartic force field (6 modes of 8 functions, 39
terms): each cycle reduces (H F_v) / ||.|| (rank 40 x 30 = 1200) back to
rank 30 for a block of 24 vectors.  Cycles 1-5 reduce from the reference's
random start (GetRandomCPvec) with 12 sweeps and their (unreduced vector,
reduction) pairs train the MLP; from cycle 6 on the MLP proposes the starts.

Checks: training lowers the loss at least fivefold; on cycles 6-8 the
proposal, after the same 3 fixed sweeps as the random start, is accepted
(residual no larger) for at least half of the vectors, and for the accepted
ones the random start needs at least one more sweep on average to reach the
accepted residual.  The measured accept rate and sweeps saved are printed.
"""
import numpy as np
import pytest

NVEC, RANK, NDOF, NB = 24, 30, 6, 8


def f_terms(batch, coef, base):
    """Each vector's F terms (base, coef) from a reduced batch."""
    out = []
    for v in range(batch.nvec):
        t0 = int(batch.term_off[v])
        out.append((base[t0:t0 + RANK].copy(), coef[t0:t0 + RANK].copy()))
    return out


def run_cycles(ws, cuda_device, ncyc=8, train_cycles=5, fixed=3, max_sweeps=12):
    import torch
    from mlcp_gb300 import als
    from mlcp_gb300 import hoplist as H
    from mlcp_gb300 import workloads as W
    from mlcp_gb300.warmstart import random_start
    hl = H.synthetic_qff(NDOF, NB, seed=2)
    rng = np.random.default_rng(0)
    F = [(rng.uniform(-0.5, 0.5, size=(RANK, NDOF * NB)), np.ones(RANK)) for _ in range(NVEC)]
    stats, losses = [], None
    for c in range(ncyc):
        batch = W.power_batch(hl, [f[0] for f in F], [f[1] for f in F], RANK)
        if c < train_cycles:
            rb = random_start(batch, seed=100 + c)
            coef = torch.from_numpy(rb.coef).to(cuda_device)
            base = torch.from_numpy(rb.base).to(cuda_device)
            st = torch.zeros(batch.nvec, dtype=torch.int32, device=cuda_device)
            als.reduce_batched(coef, base, batch.nbas, batch.rF, batch.rG, batch.term_off, max_sweeps, status=st)
            assert not st.any()
            ws.collect(batch, coef, base)
            if c == train_cycles - 1:
                losses = ws.train(epochs=300)
        else:
            coef, base, s = ws.reduce(batch, fixed_sweeps=fixed, max_sweeps=max_sweeps, seed=100 + c)
            s["cycle"] = c + 1
            stats.append(s)
        F = f_terms(batch, coef.cpu().numpy(), base.cpu().numpy())
    return losses, stats


@pytest.mark.gpu
def test_warm_start_saves_sweeps(cuda_device):
    from mlcp_gb300.warmstart import WarmStart
    ws = WarmStart(ndof=NDOF, n=NB, rank=RANK, seed=1, device=cuda_device)
    losses, stats = run_cycles(ws, cuda_device)
    print(f"training loss {losses[0]:.4e} -> {losses[-1]:.4e}")
    for s in stats:
        print(f"cycle {s['cycle']}: accept rate {s['accept_rate']:.2f}, sweeps saved {s['sweeps_saved']:.2f}, "
              f"median residual {np.median(s['residual_mlp']):.3e} (proposal) "
              f"{np.median(s['residual_random']):.3e} (random start)")
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
    acc = np.mean([s["accept_rate"] for s in stats])
    saved = np.mean([s["sweeps_saved"] for s in stats])
    assert acc >= 0.5, acc
    assert saved >= 1.0, saved
