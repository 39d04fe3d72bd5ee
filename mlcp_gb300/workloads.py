"""Seeded synthetic inputs with the shapes and value distributions of the
benchmark configurations (no dataset is involved anywhere in this path).

ALS microbenchmark (explicit-target reduction): D modes of n basis
functions, a target of rank rG with factor entries N(0,1)/sqrt(n) and weights
log-uniform in [1e-6, 1], reduced to rank rF; the starting guess is the first
rF target terms.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

ALS_SEED = 20261203


@dataclass
class AlsBatch:
    nbas: np.ndarray      # int32 [D]
    rF: np.ndarray        # int32 [nvec]
    rG: np.ndarray        # int32 [nvec]
    term_off: np.ndarray  # int64 [nvec]
    coef: np.ndarray      # float64 [nterms]
    base: np.ndarray      # float64 [nterms, nD]

    @property
    def nvec(self) -> int:
        return int(self.rF.size)

    @property
    def nD(self) -> int:
        return int(self.nbas.sum())

    def vector(self, v: int):
        """(coef, base) of vector v: F terms then G terms (copies)."""
        t0 = int(self.term_off[v])
        t1 = t0 + int(self.rF[v] + self.rG[v])
        return self.coef[t0:t1].copy(), self.base[t0:t1].copy()

    def g_bytes(self, itemsize: int = 4) -> int:
        return int(self.rG.sum()) * self.nD * itemsize


def als_batch(nvec: int, D: int, n, rF, rG, seed: int = ALS_SEED) -> AlsBatch:
    """Batch of independent reductions.  ``n`` may be an int or a per-mode
    list; ``rF``/``rG`` may be ints or per-vector lists (ragged batches)."""
    rng = np.random.default_rng(seed)
    nbas = np.full(D, n, dtype=np.int32) if np.isscalar(n) else np.asarray(n, dtype=np.int32)
    rFa = np.full(nvec, rF, dtype=np.int32) if np.isscalar(rF) else np.asarray(rF, dtype=np.int32)
    rGa = np.full(nvec, rG, dtype=np.int32) if np.isscalar(rG) else np.asarray(rG, dtype=np.int32)
    nD = int(nbas.sum())
    sizes = (rFa + rGa).astype(np.int64)
    term_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    nterms = int(sizes.sum())
    base = np.empty((nterms, nD))
    coef = np.empty(nterms)
    scale = np.repeat(1.0 / np.sqrt(nbas.astype(np.float64)), nbas)
    for v in range(nvec):
        t0, f, g = int(term_off[v]), int(rFa[v]), int(rGa[v])
        G = rng.standard_normal((g, nD)) * scale
        cg = np.exp(rng.uniform(np.log(1e-6), 0.0, g))
        base[t0 + f:t0 + f + g] = G
        coef[t0 + f:t0 + f + g] = cg
        base[t0:t0 + f] = G[:f]
        coef[t0:t0 + f] = cg[:f]
    return AlsBatch(nbas=nbas, rF=rFa, rG=rGa, term_off=term_off, coef=coef, base=base)


def main(argv=None) -> int:
    """Run one batched reduction of a seeded synthetic batch on the GPU (the
    command the profiling summaries use):
    python -m mlcp_gb300.workloads --nvec 64 --ndof 30 --nbas 12 --rf 20 --rg 3200 --sweeps 10
    python -m mlcp_gb300.workloads --svd --nvec 64 --nbas 40 --rf 16 --rg 336"""
    import argparse

    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--nvec", type=int, default=64)
    ap.add_argument("--ndof", type=int, default=30)
    ap.add_argument("--nbas", type=int, default=12)
    ap.add_argument("--rf", type=int, default=20)
    ap.add_argument("--rg", type=int, default=3200)
    ap.add_argument("--sweeps", type=int, default=10)
    ap.add_argument("--svd", action="store_true",
                    help="instead: one two-mode SVD reduction (reducsvdcpp_) of nvec vectors of rg terms on an "
                         "nbas x nbas basis to rank rf")
    a = ap.parse_args(argv)
    if a.svd:
        from mlcp_gb300 import intertwine
        rng = np.random.default_rng(ALS_SEED)
        nb = [a.nbas, a.nbas]
        base = rng.standard_normal((a.nvec * a.rg, 2 * a.nbas))
        coef = rng.uniform(0.1, 1.0, a.nvec * a.rg)
        _, _, rank = intertwine.reduc_svd(base, coef, nb, a.rg, a.rf)
        print(f"reduced {a.nvec} two-mode vectors; ranks {int(rank.min())}..{int(rank.max())}")
        return 0
    import torch

    from mlcp_gb300 import als

    dev = torch.device("cuda", 0)
    b = als_batch(a.nvec, a.ndof, a.nbas, a.rf, a.rg)
    coef = torch.from_numpy(b.coef).to(dev)
    base = torch.from_numpy(b.base).to(dev)
    status = torch.zeros(b.nvec, dtype=torch.int32, device=dev)
    als.reduce_batched(coef, base, b.nbas, b.rF, b.rG, b.term_off, a.sweeps, status=status)
    torch.cuda.synchronize()
    bad = int(status.ne(0).sum().item())
    print(f"reduced {b.nvec} vectors ({a.sweeps} sweeps); status flags on {bad}")
    return 1 if bad else 0



def apply_hamiltonian(hl, base: np.ndarray, coef: np.ndarray, shift: float = 0.0):
    """(H - shift) F as an explicit CP vector: every term t of the operator
    list applied to every term r of F (factors h_t^d F_r^d, weight alpha_t c_r),
    then the shift's copy of F (weight -shift c_r); rank (T + 1) R.  This is
    the unreduced vector that a power step reduces (reference PRODHV,
    src/MODHVECML.f90:50-209)."""
    from . import hoplist as H
    D = hl.ndof
    offs = np.concatenate([[0], np.cumsum(hl.nbas)])
    cache = H.operator_cache(hl)
    R = coef.size
    T = hl.nterms
    out_b = np.empty(((T + 1) * R, base.shape[1]))
    out_c = np.empty((T + 1) * R)
    for t in range(T):
        blk = base.copy()
        for d in range(D):
            M = cache[t][d]
            if M is not None:
                blk[:, offs[d]:offs[d + 1]] = base[:, offs[d]:offs[d + 1]] @ M.T
        out_b[t * R:(t + 1) * R] = blk
        out_c[t * R:(t + 1) * R] = hl.coef[t] * coef
    out_b[T * R:] = base
    out_c[T * R:] = -shift * coef
    return out_b, out_c


def power_batch(hl, bases, coefs, rank: int, shift: float = 0.0) -> AlsBatch:
    """A batch of power-step reductions: vector v reduces (H - shift) F_v
    (normalised to unit weight sum of squares) to rank ``rank``; its F slots
    hold the first ``rank`` target terms (to be replaced by a start)."""
    tb, tc = [], []
    for b, c in zip(bases, coefs):
        gb, gc = apply_hamiltonian(hl, b, c, shift)
        gc = gc / np.sqrt(np.sum(gc * gc))
        tb.append(gb)
        tc.append(gc)
    rG = np.array([x.size for x in tc], dtype=np.int32)
    rF = np.full(len(tc), rank, dtype=np.int32)
    sizes = (rF + rG).astype(np.int64)
    term_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
    nD = int(np.sum(hl.nbas))
    base = np.empty((int(sizes.sum()), nD))
    coef = np.empty(int(sizes.sum()))
    for v in range(len(tc)):
        t0 = int(term_off[v])
        base[t0:t0 + rank] = tb[v][:rank]
        coef[t0:t0 + rank] = tc[v][:rank]
        base[t0 + rank:t0 + rank + rG[v]] = tb[v]
        coef[t0 + rank:t0 + rank + rG[v]] = tc[v]
    return AlsBatch(nbas=np.asarray(hl.nbas, dtype=np.int32), rF=rF, rG=rG, term_off=term_off, coef=coef, base=base)


if __name__ == "__main__":
    raise SystemExit(main())
