"""Benchmark: batched explicit-target ALS rank reduction (ALS reductions/s).

Workload (the ALS microbenchmark configuration): 64 independent reductions
of random CP vectors with D=30 modes of n=12 basis functions, target rank
3200 (rank 20 x 160 Hamiltonian terms), reduced to rank 20 by 10 ALS sweeps;
factor entries N(0,1)/sqrt(12), target weights log-uniform in [1e-6, 1],
starting guess = the first 20 target terms.  Seeded synthetic data.

One step = one batched reduction of all 64 vectors (the starting guesses are
restored from a pristine copy at the start of every step).  The FP64 target
(595 MB) is larger than L2 (129 MB), so no explicit L2 flush is needed.

--impl reference times the reference's own CPU implementation of the
reduction, the Fortran host's reduc_ALS (restated in C in oracle/, OpenMP
over vectors, all host threads), on the same 64-vector workload.

Baseline legs beside the GPU measurement (never inside its timed regions):
reduc_ALS on the host cores (cpu_baseline), the FP64 oracle of the GPU
path's algorithm on a sample of the batch (whose results give the GPU's
residual errors on the headline workload: accuracy), and the
reference's own FP64 CUDA library (fp64_gpu_baseline: oracle/ref_build.py,
run in a child process on the same GPU) on a smaller sample and on one power
cycle, with the GPU's errors against it.

Further legs after the timed regions (N=1 only): the power cycle and its
neighbours (power_cycle; on the host cores the oracle of the GPU
algorithm, cpu_ms_per_cycle, and the Fortran host's own CPU solver
restated, pals_cpu_ms_per_cycle), the learned ALS warm start inside a power
iteration (warm_start: accept rate, sweeps saved, training time), and the
24-mode three-layer quartic-force-field tree solved node by node on the GPU
(tree_qff24).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NVEC, D, N, RG, RF, NALS = 64, 30, 12, 3200, 20, 10
CONFIG = {"workload": "ALS microbenchmark: 64 x (D=30, n=12, rank 3200 -> 20, 10 sweeps)",
          "batch": NVEC, "ndof": D, "nbas": N, "rank_in": RG, "rank_out": RF, "sweeps": NALS,
          "l2": "inputs larger than L2 (595 MB FP64 target per step)"}
METRIC = "ALS reductions/s"
UNIT = "reductions/s"


def max_over_ranks(x: float, dist=None, device=None) -> float:
    """The largest x over the ranks of the process group (x itself without
    one): every timing of a replicated run is the slowest rank's."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons in the background."""

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self._stop = threading.Event()
        self._proc = None
        self._thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}",
                                           "--format=csv,noheader,nounits", "-lms", "100"],
                                          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._proc = None
            return self

        def reader():
            for line in self._proc.stdout:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 7:
                    self.samples.append(parts)
        self._thread = threading.Thread(target=reader, daemon=True)
        self._thread.start()
        return self

    def stop(self):
        if self._proc is not None:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        if self._thread is not None:
            self._thread.join(timeout=5)
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        smax = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def cpu_sample_rate(batch, nvec_sample: int, threads: int, keep: bool = False):
    """Oracle (C restatement of the reference algorithm) on nvec_sample
    vectors; with keep, also the reduced (coef, base) of each vector."""
    import oracle
    coefs, bases, rfs, rgs = [], [], [], []
    for v in range(nvec_sample):
        c, b = batch.vector(v)
        coefs.append(np.ascontiguousarray(c))
        bases.append(np.ascontiguousarray(b))
        rfs.append(int(batch.rF[v]))
        rgs.append(int(batch.rG[v]))
    t0 = time.perf_counter()
    oracle.als_batched(coefs, bases, batch.nbas, rfs, rgs, NALS, nthreads=threads)
    dt = time.perf_counter() - t0
    if keep:
        return nvec_sample / dt, dt, [(coefs[v][:rfs[v]], bases[v][:rfs[v]]) for v in range(nvec_sample)]
    return nvec_sample / dt, dt


def als_errors(batch, gcoef, gbase, results):
    """Largest relative difference of the residuals ||F - G|| / ||G|| and
    largest relative distance of the reduced vectors, GPU against FP64
    results [(coef, base)] of the first len(results) vectors."""
    import oracle
    rerr, dist = 0.0, 0.0
    for v, (fc, fb) in enumerate(results):
        c0, b0 = batch.vector(v)
        f = int(batch.rF[v])
        t = int(batch.term_off[v])
        gc, gb = gcoef[t:t + f], gbase[t:t + f]
        gg = oracle.cp_dot(b0[f:], c0[f:], b0[f:], c0[f:], batch.nbas)

        def res(xc, xb):
            xx = oracle.cp_dot(xb, xc, xb, xc, batch.nbas)
            xg = oracle.cp_dot(xb, xc, b0[f:], c0[f:], batch.nbas)
            return np.sqrt(max(xx + gg - 2 * xg, 0.0) / gg)
        r_ref, r_gpu = res(fc, fb), res(gc, gb)
        rerr = max(rerr, abs(r_gpu - r_ref) / r_ref)
        aa = oracle.cp_dot(gb, gc, gb, gc, batch.nbas)
        bb = oracle.cp_dot(fb, fc, fb, fc, batch.nbas)
        ab = oracle.cp_dot(gb, gc, fb, fc, batch.nbas)
        dist = max(dist, float(np.sqrt(max(aa + bb - 2 * ab, 0.0) / bb)))
    return float(rerr), dist


FP64_SAMPLE = 4  # vectors the reference FP64 GPU library reduces (about 5 s each)


def fp64_gpu_baseline(batch, gcoef, gbase, gpu_value, cycle_gpu_ms=None):
    """The reference's own FP64 CUDA library on the same GPU: seconds per
    alscpp_ reduction on FP64_SAMPLE vectors of the batch (its residuals
    against the GPU's), and one intertwinecpp_ power cycle on the cycle
    workload (its eigenvalues against the GPU's).  None when the library is
    not built."""
    import oracle
    if not oracle.reference_built():
        return None
    out = {"kind": "reference CUDA library, FP64 build (-DUSE_DOUBLES=1), sm_103a, same GPU, child process",
           "timing": "host wall time of each entry-point call after the context exists (its device "
                     "allocations, copies, kernels, cuSOLVER solves and closing cudaDeviceReset)"}
    with oracle.Reference(timeout=1200) as ref:
        vs = list(range(FP64_SAMPLE))
        cs = np.stack([batch.vector(v)[0] for v in vs])
        bs = np.stack([batch.vector(v)[1] for v in vs])
        rc, rb, sec = ref.als(cs, bs, batch.nbas, RF, RG, NALS)
        rate = 1.0 / float(np.mean(sec))
        rerr, dist = als_errors(batch, gcoef, gbase, [(rc[k], rb[k]) for k in range(len(vs))])
        out["als"] = {"value": rate, "unit": UNIT, "seconds_per_reduction": float(np.mean(sec)),
                      "sample": f"vectors 0-{FP64_SAMPLE - 1} of the batch, one alscpp_ call each",
                      "gpu_over_fp64": gpu_value / rate, "gpu_residual_rel_err_max": rerr,
                      "gpu_vec_rel_dist_max": dist}
        if cycle_gpu_ms is not None:
            hl, Q, qc, eig0, esh = cycle_inputs()
            from mlcp_gb300 import intertwine as IT
            _, _, ge = IT.intertwine(Q, qc, hl.nbas, CYC_R, CYC_B, hl, eig0, CYC_NPOW, CYC_NALS, True, 1, esh)
            _, _, re, rsec = ref.intertwine(Q, qc, hl.nbas, CYC_R, CYC_B, hl, eig0, CYC_NPOW, CYC_NALS, True, 1,
                                            esh)
            out["power_cycle"] = {"ms_per_cycle": 1e3 * rsec, "gpu_ms_per_cycle": cycle_gpu_ms,
                                  "fp64_over_gpu_time": 1e3 * rsec / cycle_gpu_ms,
                                  "gpu_eig_rel_err_max": float(np.max(np.abs(ge - re) / np.abs(re))),
                                  "workload": "the power_cycle workload, one cycle from its seeded block"}
    return out


def reduc_sample_rate(batch, nvec_sample: int, threads: int):
    """The reference's own CPU ALS reduction (reduc_ALS, restated in the
    oracle) on nvec_sample vectors of the batch: each vector's F (its first
    rF terms) fitted to its rG target terms by NALS sweeps, OpenMP over
    vectors.  Returns (reductions/s, seconds)."""
    import oracle
    gcs, gbs, fcs, fbs = [], [], [], []
    for v in range(nvec_sample):
        c, b = batch.vector(v)
        f = int(batch.rF[v])
        gcs.append(np.ascontiguousarray(c[f:]))
        gbs.append(np.ascontiguousarray(b[f:]))
        fcs.append(np.ascontiguousarray(c[:f]).copy())
        fbs.append(np.ascontiguousarray(b[:f]).copy())
    t0 = time.perf_counter()
    oracle.reduc_als_batched(gcs, gbs, fcs, fbs, batch.nbas, NALS, nthreads=threads)
    dt = time.perf_counter() - t0
    return nvec_sample / dt, dt


REF_CPU_KIND = ("port: reduc_ALS (src/REDUCTIONML.f90:593-731), the Fortran host's CPU ALS reduction, restated in "
                "C (oracle/mlcp_oracle.c) with OpenMP over vectors")


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from mlcp_gb300 import workloads
    import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    sample = NVEC
    batch = workloads.als_batch(NVEC, D, N, RF, RG)
    for _ in range(args.warmup):
        reduc_sample_rate(batch, sample, threads)
    times = []
    for _ in range(args.steps):
        _, dt = reduc_sample_rate(batch, sample, threads)
        times.append(dt)
    total = sum(times)
    value = sample * args.steps / total
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
            "config": dict(CONFIG), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "algorithm": REF_CPU_KIND,
                             "sample": f"all {NVEC} vectors per step, full {NALS} sweeps each"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# Power cycle (intertwinecpp_): Henon-Heiles with the config-1 shape at its
# 6-mode level (10 HO functions per mode, lambda = 0.111803), rank 16, a
# block of 40 vectors, npow = nals = 10, update on.
CYC_D, CYC_N, CYC_R, CYC_B, CYC_NPOW, CYC_NALS = 6, 10, 16, 40, 10, 10
# Two-mode node (40 x 40 functions, as the upper layers of a mode tree
# combine 40-state modes); SVD reductions of 64 vectors of 16 x (20 + 1)
# terms (the size of (H - E) v for a 20-term H).
SVD_NBAS, SVD_T, SVD_NVEC = [40, 40], 20, 64
# Pre-diagonalisation of a two-mode node whose block is all its product
# functions (12 x 12 = 144 vectors: the solver's direct-diagonalisation case).
DIAG_N = 12
# Power cycles of the solver loop measured to convergence against Lanczos.
SOLVE_CYCLES = 60


def diag_product_block(n, rk):
    """Every product function of an n x n node as a rank-1 vector padded to
    rank rk with zero weights."""
    B = n * n
    base = np.zeros((B * rk, 2 * n))
    coef = np.zeros(B * rk)
    for a in range(n):
        for b in range(n):
            i = a * n + b
            base[i * rk, a] = 1.0
            base[i * rk, n + b] = 1.0
            coef[i * rk] = 1.0
    return base, coef, B


def cycle_inputs(seed=20261203):
    from mlcp_gb300 import hoplist as H
    hl = H.henon_heiles(D=CYC_D, n=CYC_N, lam=0.111803)
    rng = np.random.default_rng(seed)
    Q = rng.uniform(-0.5, 0.5, size=(CYC_R * CYC_B, CYC_D * CYC_N))
    qc = np.ones(CYC_R * CYC_B)
    # shift from harmonic estimates: E ~ 3 + (number of quanta)
    eig0 = 3.0 + np.sort(np.concatenate([[0], np.ones(6), 2 * np.ones(21), 3 * np.ones(56)]))[:CYC_B]
    esh = 0.5 * (2 * eig0[-1] - eig0[-2] + (3.0 + 9 * CYC_D))
    return hl, Q, qc, eig0, esh


def run_cycle_bench(steps: int, cpu: bool):
    """GPU power-cycle time through the C ABI (host buffers in and out, as
    the Fortran host calls it) and the oracle's time for one cycle on the host
    cores.  No eigenvalue comparison is reported here: one cycle from a random
    block is far from converged and its Ritz values move by several percent
    under any rounding-level change (the FP64 oracle itself moves 9% between
    the FP64- and FP32-build penalty rules on this workload); the cycle's
    parity is checked in the GPU tests on well-posed cases."""
    from mlcp_gb300 import intertwine as IT
    hl, Q, qc, eig0, esh = cycle_inputs()
    IT.intertwine(Q, qc, hl.nbas, CYC_R, CYC_B, hl, eig0, CYC_NPOW, CYC_NALS, True, 1, esh)  # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        gb, gc, ge = IT.intertwine(Q, qc, hl.nbas, CYC_R, CYC_B, hl, eig0, CYC_NPOW, CYC_NALS, True, 1, esh)
    gpu_ms = 1e3 * (time.perf_counter() - t0) / steps
    out = {"workload": f"Henon-Heiles D={CYC_D} n={CYC_N}, rank {CYC_R}, block {CYC_B}, npow={CYC_NPOW}, "
                       f"nals={CYC_NALS}, update on", "gpu_ms_per_cycle": gpu_ms}
    # the update = F step's Rayleigh quotients of the block (getqhqdiagcpp_)
    IT.qhq_diag(gb, gc, hl.nbas, CYC_R, CYC_B, hl)
    t0 = time.perf_counter()
    for _ in range(steps):
        IT.qhq_diag(gb, gc, hl.nbas, CYC_R, CYC_B, hl)
    out["qhq_diag_gpu_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    # GetSpectralRange before a node's solve (getspectralrangecpp_): two
    # vectors, npow power steps per round, 10 rounds
    import oracle
    sb, sc = oracle.spectral_start(hl.nbas, CYC_R, seed=7)
    IT.spectral_range(sb, sc, hl.nbas, CYC_R, hl, CYC_NPOW, 10)
    t0 = time.perf_counter()
    for _ in range(steps):
        _, _, bounds = IT.spectral_range(sb, sc, hl.nbas, CYC_R, hl, CYC_NPOW, 10)
    out["spectral_range_gpu_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    # the next layer's operator update (updateopermatcpp_): three operators of mode 1
    rng = np.random.default_rng(11)
    xm = []
    for _ in range(3):
        X = rng.normal(size=(CYC_N, CYC_N))
        X = X + X.T
        xm.append([X[i, j] for j in range(CYC_N) for i in range(j + 1)])
    xm = np.array(xm)
    IT.update_opermat(1, gb, gc, hl.nbas, CYC_R, CYC_B, xm)
    t0 = time.perf_counter()
    for _ in range(steps):
        IT.update_opermat(1, gb, gc, hl.nbas, CYC_R, CYC_B, xm)
    out["update_opermat_gpu_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    out["spectral_range"] = [float(bounds[0]), float(bounds[1])]
    # two-mode nodes: GetSpectralRange as the solver calls it (rank 16,
    # npow 10, 5 rounds) on a 40 x 40 two-mode quartic force field, and a
    # batch of 64 SVD reductions of 336-term vectors to 16 terms
    from mlcp_gb300 import hoplist as H
    h2 = H.synthetic_qff(2, SVD_NBAS[0], seed=5)
    tb, tc = oracle.spectral_start(h2.nbas, CYC_R)
    IT.spectral_range(tb, tc, h2.nbas, CYC_R, h2, CYC_NPOW, 5)
    t0 = time.perf_counter()
    for _ in range(steps):
        _, _, b2 = IT.spectral_range(tb, tc, h2.nbas, CYC_R, h2, CYC_NPOW, 5)
    out["spectral_range_2mode_gpu_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    out["spectral_range_2mode"] = [float(b2[0]), float(b2[1])]
    rg = CYC_R * (SVD_T + 1)
    srng = np.random.default_rng(13)
    svb = srng.normal(size=(SVD_NVEC * rg, sum(SVD_NBAS)))
    svc = srng.uniform(0.1, 1.0, SVD_NVEC * rg)
    IT.reduc_svd(svb, svc, SVD_NBAS, rg, CYC_R)
    t0 = time.perf_counter()
    for _ in range(steps):
        IT.reduc_svd(svb, svc, SVD_NBAS, rg, CYC_R)
    out["reduc_svd_gpu_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    out["workload_2mode"] = (f"two-mode quartic force field {SVD_NBAS[0]}x{SVD_NBAS[1]} ({h2.nterms} terms), "
                             f"rank {CYC_R}; reduc_svd: {SVD_NVEC} vectors of {rg} terms -> {CYC_R}")
    # pre-diagonalisation (diagonalizecpp_): a two-mode node whose block is
    # every product function (the solver's diag case, 12 x 12 = 144 states),
    # and the 40-vector Henon-Heiles block with ALS updates
    hd = H.synthetic_qff(2, DIAG_N, seed=6)
    db, dc, nbd = diag_product_block(DIAG_N, CYC_R)
    IT.diagonalize(db, dc, hd.nbas, CYC_R, nbd, hd, 0)
    t0 = time.perf_counter()
    for _ in range(steps):
        IT.diagonalize(db, dc, hd.nbas, CYC_R, nbd, hd, 0)
    out["diagonalize_2mode_gpu_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    IT.diagonalize(gb, gc, hl.nbas, CYC_R, CYC_B, hl, CYC_NALS)
    t0 = time.perf_counter()
    for _ in range(steps):
        IT.diagonalize(gb, gc, hl.nbas, CYC_R, CYC_B, hl, CYC_NALS)
    out["diagonalize_hh6_gpu_ms"] = 1e3 * (time.perf_counter() - t0) / steps
    # the solver loop to convergence (SolveHPsi with the GPU cycle): 60
    # cycles from the product-function guess, eigenvalues against the
    # Lanczos values of the full 10^6 basis
    from mlcp_gb300 import solver
    t0 = time.perf_counter()
    _, _, seig, _, shist = solver.solve(hl, CYC_B, CYC_R, SOLVE_CYCLES, CYC_NPOW, CYC_NALS)
    s_sec = time.perf_counter() - t0
    with open(os.path.join(ROOT, "tests", "golden", "hh6_n10_lowest40.json")) as f:
        ex = np.array(json.load(f)["eigenvalues"])
    serr = seig - ex
    out["solver"] = {"cycles": SOLVE_CYCLES, "seconds": s_sec, "e0_abs_error": float(serr[0]),
                     "max_abs_error_0_1_quanta": float(np.abs(serr[:7]).max()),
                     "max_abs_error_0_2_quanta": float(np.abs(serr[:28]).max()),
                     "max_abs_error_all_40": float(np.abs(serr).max()), "last_rms_change": shist[-1],
                     "reference": "ARPACK Lanczos, full 10^6 basis (tests/golden/hh6_n10_lowest40.json)"}
    # the benchmark's whole tree (three two-mode nodes of 30 states, a
    # three-mode top layer of 40 states; ncycle = npow = nals = 10, rank 16),
    # every solve and operator update on the GPU, against the same Lanczos values
    from mlcp_gb300 import tree
    t0 = time.perf_counter()
    teig, tinfo = tree.hh_tree(D=CYC_D, n=CYC_N, keep=30, top_nev=CYC_B, rk=CYC_R, ncycle=10, npow=CYC_NPOW,
                               nals=CYC_NALS)
    terr = teig - ex
    out["tree"] = {"workload": "Henon-Heiles D=6 n=10, tree (0 1)(2 3)(4 5) keeping 30 states each / top 40 states, "
                               "rank 16, ncycle=npow=nals=10", "seconds": time.perf_counter() - t0,
                   "e0_abs_error": float(terr[0]), "max_abs_error_0_1_quanta": float(np.abs(terr[:7]).max()),
                   "max_abs_error_0_2_quanta": float(np.abs(terr[:28]).max()),
                   "max_abs_error_all_40": float(np.abs(terr).max()),
                   "reference": "ARPACK Lanczos, full 10^6 basis (tests/golden/hh6_n10_lowest40.json)"}
    out["workload_diagonalize"] = (f"two-mode quartic force field {DIAG_N}x{DIAG_N}, all {nbd} product functions, "
                                   f"rank {CYC_R}; Henon-Heiles block as the cycle with nals={CYC_NALS}")
    if cpu:
        t0 = time.perf_counter()
        oracle.intertwine(Q, qc, hl.nbas, CYC_R, CYC_B, hl, eig0, CYC_NPOW, CYC_NALS, True, 1, esh)
        out["cpu_ms_per_cycle"] = 1e3 * (time.perf_counter() - t0)
        # the Fortran host's own CPU solver (solver pals, lowmem 4: ALS_POW3,
        # ALS_ORTHO_2, PRODHV_ALS2, ALS_SUMLCVEC_2) restated, OpenMP as there
        t0 = time.perf_counter()
        oracle.pals_cycle(Q, qc, hl.nbas, CYC_R, CYC_B, hl, eig0, CYC_NPOW, CYC_NALS, True, 1, esh)
        out["pals_cpu_ms_per_cycle"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        pb, pc = oracle.pals_pow3(Q, qc, hl.nbas, CYC_R, CYC_B, hl, CYC_NPOW, 1, esh)
        t1 = time.perf_counter()
        pb, pc = oracle.pals_ortho2(pb, pc, hl.nbas, CYC_R, CYC_B, CYC_NALS)
        t2 = time.perf_counter()
        oracle.pals_diagonalize(pb, pc, hl.nbas, CYC_R, CYC_B, hl, CYC_NALS)
        t3 = time.perf_counter()
        out["pals_cpu_stage_ms"] = {"ALS_POW3": 1e3 * (t1 - t0), "ALS_ORTHO_2": 1e3 * (t2 - t1),
                                    "Diagonalize": 1e3 * (t3 - t2)}
        # the same solver at lowmem 3 (ALS_ORTHO_3, PRODHV_ALS3, ALS_SUMLCVEC_3: no stored PS)
        t0 = time.perf_counter()
        oracle.pals_cycle(Q, qc, hl.nbas, CYC_R, CYC_B, hl, eig0, CYC_NPOW, CYC_NALS, True, 1, esh, lowmem=3)
        out["pals_lowmem3_cpu_ms_per_cycle"] = 1e3 * (time.perf_counter() - t0)
        out["cpu_threads"] = os.cpu_count()
        t0 = time.perf_counter()
        oracle.qhq_diag(gb, gc, hl.nbas, CYC_R, CYC_B, hl)
        out["qhq_diag_cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.spectral_range(sb, sc, hl.nbas, CYC_R, hl, CYC_NPOW, 10)
        out["spectral_range_cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.update_opermat(1, gb, gc, hl.nbas, CYC_R, CYC_B, xm)
        out["update_opermat_cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.spectral_range_2mode(h2.nbas, CYC_R, h2, CYC_NPOW, 5)
        out["spectral_range_2mode_cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        for v in range(SVD_NVEC):
            oracle.reduc_svd(svb[v * rg:(v + 1) * rg], svc[v * rg:(v + 1) * rg], SVD_NBAS, CYC_R)
        out["reduc_svd_cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        t0 = time.perf_counter()
        oracle.diagonalize_dense(db, dc, hd.nbas, CYC_R, nbd, hd)
        out["diagonalize_2mode_cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        out["cpu_cores"] = os.cpu_count()
        out["cpu_kind"] = "port"
    return out


# Learned warm start inside a power iteration: a 6-mode quartic force field
# of 8 functions per mode, 24 vectors of rank 30, (H - 30000) F reduced back
# to rank 30 each cycle; cycles 1-5 train, 6-8 are tested.
WS_D, WS_N, WS_RANK, WS_NVEC, WS_SHIFT = 6, 8, 30, 24, 30000.0


def run_warm_start_bench(dev):
    """Accept rate and sweeps saved by the MLP's proposals against the
    reference's random start (the yardstick of the acceptance test), and the
    on-GPU training time."""
    from mlcp_gb300 import hoplist as H
    from mlcp_gb300.warmstart import WarmStart, power_steps
    ws = WarmStart(ndof=WS_D, n=WS_N, rank=WS_RANK, seed=1, device=dev)
    hl = H.synthetic_qff(WS_D, WS_N, seed=2)
    t0 = time.perf_counter()
    losses, stats, t_train = power_steps(ws, hl, nvec=WS_NVEC, shift=WS_SHIFT)
    return {"workload": f"synthetic QFF D={WS_D} n={WS_N}: {WS_NVEC} vectors, (H - {WS_SHIFT:g}) F of rank "
                        f"{WS_RANK} x {hl.nterms} reduced to rank {WS_RANK}; cycles 1-5 train, 6-8 tested",
            "network": "3 layers, width 256, BF16 weights, FP32 accumulation (tcgen05)",
            "train_seconds": t_train, "loss_first": float(losses[0]), "loss_last": float(losses[-1]),
            "accept_rate": float(np.mean([s["accept_rate"] for s in stats])),
            "sweeps_saved": float(np.mean([s["sweeps_saved"] for s in stats])),
            "per_cycle": [{"cycle": s["cycle"], "accept_rate": float(s["accept_rate"]),
                           "sweeps_saved": float(s["sweeps_saved"])} for s in stats],
            "seconds": time.perf_counter() - t0}


def run_tree3_bench():
    """The three-layer tree of the 24-mode quartic force field (pairs, groups
    of four, top node), every node solved by the GPU solver loop."""
    from mlcp_gb300 import tree
    t0 = time.perf_counter()
    eig, info = tree.qff_tree(D=24, n=8, seed=3, keep_pair=24, keep_group=48, top_nev=100, rk=30, ncycle=10,
                              npow=15, nals=15)
    top = info["layers"][-1][0]
    return {"workload": "synthetic QFF D=24, n=8: pairs (24 states) -> groups of four (48 states) -> top "
                        "(100 states), rank 30, ncycle=10, npow=nals=15",
            "seconds": time.perf_counter() - t0, "top_terms": top["terms"], "lowest": [float(x) for x in eig[:5]],
            "top_last_rms": top["last_rms"]}


def run_gpu(args):
    import torch
    from mlcp_gb300 import _lib, als, workloads

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    L = _lib.load()
    batch = workloads.als_batch(NVEC, D, N, RF, RG, seed=workloads.ALS_SEED + rank)
    coef0 = torch.from_numpy(batch.coef).to(dev)
    base0 = torch.from_numpy(batch.base).to(dev)
    coef = coef0.clone()
    base = base0.clone()
    status = torch.zeros(NVEC, dtype=torch.int32, device=dev)
    # F rows of every vector (restored from the pristine copy each step)
    f_rows = torch.cat([torch.arange(int(t), int(t) + RF) for t in batch.term_off]).to(dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        base.index_copy_(0, f_rows, base0.index_select(0, f_rows))
        coef.index_copy_(0, f_rows, coef0.index_select(0, f_rows))
        als.reduce_batched(coef, base, batch.nbas, batch.rF, batch.rG, batch.term_off, NALS, status=status,
                           stream=stream)

    def barrier():
        if dist is not None:
            dist.barrier()

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    assert not status.any().item(), "non-positive-definite normal equations in warm-up"

    # device-resident timing
    clocks = ClockSampler(local).start() if rank == 0 else None
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop() if clocks else None
    ms = max_over_ranks(ms, dist, dev)
    value = NVEC * ws * args.steps / (ms / 1e3)

    # dominant-kernel timing (cluster ALS kernel) on the launching stream
    L.mlcp_gb300_set_kernel_timing(1)
    kms = []
    for _ in range(args.steps):
        step()
        kms.append(L.mlcp_gb300_last_kernel_ms())
    L.mlcp_gb300_set_kernel_timing(0)
    kernel_ms = float(np.mean(kms))
    torch.cuda.synchronize()
    gcoef, gbase = coef.cpu().numpy(), base.cpu().numpy()  # the last step's reduced batch
    alg_bytes = NALS * batch.g_bytes(4)  # FP32 target slice streamed once per mode visit
    peak, peak_kind = measured_peak_hbm()
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9

    # end to end through the host-buffer C entry point (pinned host memory)
    hcoef = torch.from_numpy(batch.coef.copy()).pin_memory()
    hbase = torch.from_numpy(batch.base.copy()).pin_memory()
    hc, hb = hcoef.numpy(), hbase.numpy()
    f_slices = [slice(int(t), int(t) + RF) for t in batch.term_off]

    def e2e_step():
        for sl in f_slices:  # each vector's starting guess, restored in place
            hb[sl] = batch.base[sl]
            hc[sl] = batch.coef[sl]
        als.reduce_batched_host(hc, hb, batch.nbas, batch.rF, batch.rG, batch.term_off, NALS)
    for _ in range(2):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_s = max_over_ranks(e2e_s, dist, dev)
    h2d = int(batch.coef.nbytes + batch.base.nbytes)
    d2h = int(NVEC * RF * (batch.nD + 1) * 8)
    e2e_value = NVEC * ws * args.steps / e2e_s

    traffic = None
    tpath = os.path.join(ROOT, "profiles", "als_cluster_kernel_traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get("bytes_per_launch")

    # CPU baseline: the oracle on a bounded sample (rank 0, N=1 only)
    cpu = None
    accuracy = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, dt = reduc_sample_rate(batch, NVEC, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "algorithm": REF_CPU_KIND,
               "sample": f"all {NVEC} vectors (full {NALS} sweeps each) in {dt:.1f} s"}
        # accuracy against the FP64 oracle of the GPU path's own algorithm (ITERATE_ALS)
        sample = min(NVEC, threads)
        _, _, fp64 = cpu_sample_rate(batch, sample, threads, keep=True)
        rerr, vdist = als_errors(batch, gcoef, gbase, fp64)
        accuracy = {"against": "FP64 oracle (the reference's algorithm; pinned to the reference library by "
                               "tests/test_gpu_reference.py)", "sample": f"vectors 0-{sample - 1}",
                    "als_residual_rel_err_max": rerr, "als_vec_rel_dist_max": vdist}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32+dw48", "data": "synthetic (seeded)",
                "dtype_note": "FP32 contractions with FP32 accumulation; normal equations, solves and norms in "
                              "double-word FP32 pairs (~48-bit significand, FP32 exponent range); FP64 in and out",
                "config": dict(CONFIG),
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "note": "alscpp_ keeps the target on the host: its FP64 copy crosses the host link every "
                                "step, read by the GPU from mapped pinned memory"},
                "accuracy": accuracy,
                "gpu_launches": 3 * args.steps,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                             "kernel": "als_cluster_kernel", "kernel_ms": kernel_ms,
                             "algorithmic_bytes": alg_bytes},
                "cpu_baseline": cpu, "clocks": clk,
                "autotune": _lib.autotune_report().strip().splitlines()}
        if not args.no_cycle and ws == 1:
            line["power_cycle"] = run_cycle_bench(max(1, min(args.steps, 5)), cpu=not args.no_cpu)
        if not args.no_warm_start and ws == 1:
            line["warm_start"] = run_warm_start_bench(dev)
        if not args.no_tree3 and ws == 1:
            line["tree_qff24"] = run_tree3_bench()
        if not args.no_fp64 and ws == 1:
            cyc_ms = line["power_cycle"]["gpu_ms_per_cycle"] if "power_cycle" in line else None
            line["fp64_gpu_baseline"] = fp64_gpu_baseline(batch, gcoef, gbase, e2e_value, cyc_ms)
        line["autotune"] = _lib.autotune_report().strip().splitlines()  # with the legs' Gram-Schmidt shapes
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline sample")
    ap.add_argument("--no-cycle", action="store_true", help="skip the power-cycle measurement")
    ap.add_argument("--no-fp64", action="store_true",
                    help="skip the reference FP64 GPU library's timing (fp64_gpu_baseline)")
    ap.add_argument("--no-warm-start", action="store_true", help="skip the learned warm-start measurement")
    ap.add_argument("--no-tree3", action="store_true", help="skip the 24-mode three-layer tree")
    ap.add_argument("--cycle-only", action="store_true",
                    help="time only the power cycle (--steps cycles after one warm-up) and print its JSON")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.cycle_only:
        print(json.dumps(run_cycle_bench(max(1, args.steps), cpu=not args.no_cpu)), flush=True)
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
