"""The learned ALS warm start (mlcp_gb300/warmstart.py) inside a power
iteration of a synthetic quartic force field (6 modes of 8 functions, 39
terms): each cycle reduces (H - 30000) F_v / ||.|| (rank 40 x 30 = 1200) back
to rank 30 for a block of 24 vectors.  Cycles 1-5 are the solver's own
reductions (each from the vector's previous iterate, 20 sweeps) and their
(unreduced vector, reduction) pairs train the MLP (600 full-batch Adam
steps); from cycle 6 on the MLP proposes the starts and the reference's
random start (GetRandomCPvec) runs beside it as the fallback and the yardstick.

Checks: training lowers the loss at least fivefold; over cycles 6-8 the
proposal, after the same 3 fixed sweeps as the random start, is accepted
(residual no larger) for at least 75 % of the vectors, and for the accepted
ones the random start needs on average at least 1.5 more sweeps to reach the
accepted residual (measured on the GB300: accept rates 0.92-1.0, 2.0-3.4
sweeps saved).  The measured values are printed.
"""
import numpy as np
import pytest


@pytest.mark.gpu
def test_warm_start_saves_sweeps(cuda_device):
    from mlcp_gb300 import hoplist as H
    from mlcp_gb300.warmstart import WarmStart, power_steps
    ws = WarmStart(ndof=6, n=8, rank=30, seed=1, device=cuda_device)
    hl = H.synthetic_qff(6, 8, seed=2)
    losses, stats, t_train = power_steps(ws, hl, nvec=24, shift=30000.0)
    print(f"training loss {losses[0]:.4e} -> {losses[-1]:.4e} in {t_train:.2f} s")
    for s in stats:
        print(f"cycle {s['cycle']}: accept rate {s['accept_rate']:.2f}, sweeps saved {s['sweeps_saved']:.2f}, "
              f"median residual {np.median(s['residual_mlp']):.3e} (proposal) "
              f"{np.median(s['residual_random']):.3e} (random start)")
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
    acc = np.mean([s["accept_rate"] for s in stats])
    saved = np.mean([s["sweeps_saved"] for s in stats])
    assert acc >= 0.75, acc
    assert saved >= 1.5, saved
