// ALS-guided Gram-Schmidt over a block of CP vectors (reference GramSchmidt,
// src/intertw_lcv.cu:131-205, with lcv_build_linear_system :77-127).
//
// Vector iv (iv >= 1) is fitted, mode by mode, to
//   F - sum_{k<iv} <Q_k, F> Q_k,
// where F is its current iterate and the coefficients <Q_k, F> are
// recomputed at every mode step (gramsumoverrow + sumarray in the reference).
// The pairwise per-mode overlaps P_k,d(r,i) = <Q_k,r^d, F_i^d> are kept and
// only the mode just solved is refreshed, so a mode step costs
// O(iv R^2 (D + 2n)) instead of rebuilding every product over all modes.
//
// Precision.  Once power iteration has made the block's vectors nearly
// parallel, the target F - sum_k <Q_k,F> Q_k is a small difference of large
// terms, and FP32 contractions lose it to cancellation; the reference runs
// this stage in FP64.  GB300 issues FP64 at a small fraction of its FP32
// rate, so everything here runs in double-word arithmetic (dword.cuh: about
// 48-bit significands on the FP32 pipes).  The R x R normal equations are
// solved by an FP32 Gauss-Jordan inverse with double-word iterative
// refinement, falling back to a double-word LDL^T (dwsolve.cuh).
//
// GB300 layout: the loop over vectors is sequential, but within a mode step
// the work over the earlier vectors k is independent.  One thread-block
// cluster of up to 16 CTAs runs the whole orthogonalisation in one launch;
// CTA `rank` owns the earlier vectors k = rank (mod cluster) and keeps their
// factors, weights and overlaps resident in its shared memory (its global
// scratch when they do not fit).  Each CTA computes its vectors' products,
// coefficients and right-hand-side contributions; the partial right-hand
// sides meet through distributed shared memory, and every CTA runs the same
// small solve on the same data, so each holds the identical new factor and
// nothing is broadcast back.  One cluster barrier per mode step.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "dword.cuh"
#include "dwsolve.cuh"
#include "fastdiv.cuh"
#include "intertwine.cuh"

namespace cg = cooperative_groups;

namespace mlcp {

namespace {

constexpr int kGsThreads = 512;
constexpr int kGsWarps = kGsThreads / 32;
static_assert(kGsWarps == 16, "block_sum reduces 16 warp partials");

// Groups of arrays that move to global scratch (in this order) when shared
// memory cannot hold them.
enum : int { kGroupQ = 1, kGroupP = 2, kGroupF = 4, kGroupAll = 7 };

struct GsDims {
  int R, D, nD, npm, nkmax, gmask;
};

struct GsArrays {
  dw *qf, *qw, *qc;        // [nkmax][R][nD] owned vectors' factors, the same times their weights; [nkmax][R] weights
  dw *P, *psn, *ppsn, *part;  // [nkmax][D][R*R] overlaps (index r*R+i); [nkmax][R*R] products over d != j,
                               // and over d not in {j, next mode}; [nkmax+1][2][R*npm] partial dot products
  dw *fb, *g;              // [R][nD] vector being fitted; [D][R*R] its Grams
  dw *fcs, *wf, *Gp, *pGp, *BB, *gpart, *gco, *bpart, *X, *b0, *res, *dinv, *u, *red, *misc;
  float *gi, *rred;
  dwsolve::ColScratch cs;
  int *nb, *off, *flags;
  FastDiv* fd;  // divisors of the step's index splits: R, R*R, RRp, then R*n_d per mode
};

// Entries of R*R rounded up to whole warps.
__host__ __device__ inline int gs_rrp(int R) { return (R * R + 31) / 32 * 32; }

// Assigns the arrays (null bases: sizes only).  Returns the shared-memory
// bytes; *gwork receives the global scratch entries (dw) of one CTA.
__host__ __device__ inline size_t gs_carve(const GsDims& m, GsArrays* a, unsigned char* sbase, dw* gbase,
                                           size_t* gwork) {
  const int R = m.R, nkm = m.nkmax;
  const size_t RR = (size_t)R * R, Rn = (size_t)R * m.npm;
  size_t so = 0, go = 0;
  auto take_s = [&](size_t bytes) -> unsigned char* {
    const size_t r = so;
    so += (bytes + 15) / 16 * 16;
    return sbase ? sbase + r : nullptr;
  };
  auto take = [&](int group, size_t n) -> dw* {
    if (m.gmask & group) {
      const size_t r = go;
      go += (n + 1) / 2 * 2;
      return gbase ? gbase + r : nullptr;
    }
    return (dw*)take_s(sizeof(dw) * n);
  };
  a->qf = take(kGroupQ, (size_t)nkm * R * m.nD);
  a->qw = take(kGroupQ, (size_t)nkm * R * m.nD);
  a->qc = take(kGroupQ, (size_t)nkm * R);
  a->P = take(kGroupP, (size_t)nkm * m.D * RR);
  a->psn = take(kGroupP, (size_t)nkm * RR);
  a->ppsn = take(kGroupP, (size_t)nkm * RR);
  a->part = take(kGroupP, (size_t)(nkm + 1) * 2 * Rn);
  a->fb = take(kGroupF, (size_t)R * m.nD);
  a->g = take(kGroupF, (size_t)m.D * RR);
  a->fcs = (dw*)take_s(sizeof(dw) * R);
  a->wf = (dw*)take_s(sizeof(dw) * Rn);
  a->Gp = (dw*)take_s(sizeof(dw) * RR);
  a->pGp = (dw*)take_s(sizeof(dw) * RR);
  a->BB = (dw*)take_s(sizeof(dw) * RR);
  a->gpart = (dw*)take_s(sizeof(dw) * nkm * (gs_rrp(R) / 32));
  a->gco = (dw*)take_s(sizeof(dw) * nkm);
  a->bpart = (dw*)take_s(sizeof(dw) * 2 * Rn);
  a->X = (dw*)take_s(sizeof(dw) * Rn);
  a->b0 = (dw*)take_s(sizeof(dw) * Rn);
  a->res = (dw*)take_s(sizeof(dw) * Rn);
  a->dinv = (dw*)take_s(sizeof(dw) * R);
  a->u = (dw*)take_s(sizeof(dw) * R);
  a->red = (dw*)take_s(sizeof(dw) * kGsWarps);
  a->misc = (dw*)take_s(sizeof(dw) * 4);
  a->gi = (float*)take_s(sizeof(float) * 2 * RR);
  a->rred = (float*)take_s(sizeof(float) * 4);
  a->cs.conv = (float*)take_s(sizeof(float) * 64);
  a->cs.rmax = (float*)take_s(sizeof(float) * 16 * 32);
  a->cs.rsum = (dw*)take_s(sizeof(dw) * 16 * 32);
  a->nb = (int*)take_s(sizeof(int) * (m.D + 1));
  a->off = (int*)take_s(sizeof(int) * (m.D + 1));
  a->flags = (int*)take_s(sizeof(int) * 4);
  a->fd = (FastDiv*)take_s(sizeof(FastDiv) * (m.D + 3));
  if (gwork) *gwork = go;
  return so;
}

__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// Threads outside the solver team (warps 4-15).
constexpr int kWorkerThreads = kGsThreads - dwsolve::kSolverThreads;
// Barrier of the threads w0..511 (named barrier 2).
__device__ __forceinline__ void worker_sync(int w0) {
  asm volatile("bar.sync 2, %0;" ::"r"(kGsThreads - w0) : "memory");
}

// Sum over the block; every thread gets the same value (dw_add is
// commutative, so the butterflies agree across lanes and warps).
__device__ dw block_sum(dw v, dw* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = dw_add(v, dwsolve::dw_shfl_xor(v, o));
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  dw s = red[lane & (kGsWarps - 1)];
  for (int o = kGsWarps / 2; o > 0; o >>= 1) s = dw_add(s, dwsolve::dw_shfl_xor(s, o));
  return s;
}

// block_sum without its leading barrier, for callers after which no thread
// can still be reading red from an earlier sum (many barriers since).
__device__ dw block_sum_ready(dw v, dw* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = dw_add(v, dwsolve::dw_shfl_xor(v, o));
  if (lane == 0) red[warp] = v;
  __syncthreads();
  dw s = red[lane & (kGsWarps - 1)];
  for (int o = kGsWarps / 2; o > 0; o >>= 1) s = dw_add(s, dwsolve::dw_shfl_xor(s, o));
  return s;
}

struct Gs {
  GsArrays a;
  int R, RR, RRp, D, nD, npm, CL, rank, tid;
  int G, cid, gr, NC;  // clusters, this CTA's cluster, its index over all CTAs, all CTAs
  int rv;  // rank of the vector being fitted (ragged blocks; R otherwise)
};

// Ragged ranks: rows and columns >= rv of the normal equations are the
// identity, so the padded terms stay decoupled from the fit.
__device__ __forceinline__ dw mask_bb(const Gs& c, int i, int i2, dw v) {
  return (i >= c.rv || i2 >= c.rv) ? dw_make(i == i2 ? 1.f : 0.f) : v;
}

// The vector iv as the working copy: factors, weights, penalty.
__device__ void load_vector(const Gs& c, const GsParams& p, int iv) {
  const double* fb = p.base + (size_t)iv * c.R * c.nD;
  for (int e = c.tid; e < c.R * c.nD; e += kGsThreads) c.a.fb[e] = dw_from_double(fb[e]);
  for (int i = c.tid; i < c.R; i += kGsThreads) c.a.fcs[i] = dw_from_double(p.coef[(size_t)iv * c.R + i]);
  if (c.tid == 0) {
    double pen = p.coef[(size_t)iv * c.R];
    for (int i = 1; i < c.R; ++i) pen = fmax(pen, p.coef[(size_t)iv * c.R + i]);
    c.a.misc[0] = dw_from_double(pen * 1.0e-10);  // FP64-build rule of the reference for this stage
  }
  __syncthreads();
}

// Grams of the working vector, every mode (symmetric, both triangles stored).
__device__ void all_grams(const Gs& c) {
  const int R = c.R, RR = c.RR;
  for (int e = c.tid; e < c.D * RR; e += kGsThreads) {
    const int d = e / RR, ee = e - d * RR, i = ee % R, i2 = ee / R;
    if (i > i2) continue;
    const dw* x = c.a.fb + (size_t)i * c.nD + c.a.off[d];
    const dw* y = c.a.fb + (size_t)i2 * c.nD + c.a.off[d];
    dw_acc acc = acc_zero();
    for (int q = 0; q < c.a.nb[d]; ++q) acc_fma(acc, x[q], y[q]);
    const dw s = acc_value(acc);
    c.a.g[(size_t)d * RR + i + i2 * R] = s;
    c.a.g[(size_t)d * RR + i2 + i * R] = s;
  }
  __syncthreads();
}

// Overlaps of the owned earlier vectors with the working vector, every mode.
__device__ void all_overlaps(const Gs& c, int nk) {
  const int R = c.R, RR = c.RR, DRR = c.D * RR;
  for (int e = c.tid; e < nk * DRR; e += kGsThreads) {
    const int kl = e / DRR, rem = e - kl * DRR, d = rem / RR, ee = rem - d * RR, r = ee / R, i = ee - r * R;
    const dw* x = c.a.qf + ((size_t)kl * R + r) * c.nD + c.a.off[d];
    const dw* y = c.a.fb + (size_t)i * c.nD + c.a.off[d];
    dw_acc acc = acc_zero();
    for (int q = 0; q < c.a.nb[d]; ++q) acc_fma(acc, x[q], y[q]);
    c.a.P[(size_t)kl * DRR + rem] = acc_value(acc);
  }
  __syncthreads();
}

// Weights divided by sqrt(<F,F>).
__device__ void normalize_weights(const Gs& c) {
  const int R = c.R;
  dw part = dw_make(0.f);
  for (int e = c.tid; e < c.RR; e += kGsThreads) {
    dw prod = dw_mul(c.a.fcs[e % R], c.a.fcs[e / R]);
    for (int d = 0; d < c.D; ++d) prod = dw_mul(prod, c.a.g[(size_t)d * c.RR + e]);
    part = dw_add(part, prod);
  }
  const dw q = dw_sqrt(dw_abs(block_sum(part, c.a.red)));
  __syncthreads();  // every thread has read fcs
  for (int i = c.tid; i < R; i += kGsThreads) c.a.fcs[i] = dw_div(c.a.fcs[i], q);
  __syncthreads();
}

// The finished vector: FP64 output (CTA 0 of the grid), and the owner's
// resident copy when later vectors use it.
__device__ void finish_vector(const Gs& c, const GsParams& p, int iv, bool factors) {
  const int R = c.R, nD = c.nD;
  if (c.gr == 0) {
    double* fb = p.base + (size_t)iv * R * nD;
    if (factors)
      for (int e = c.tid; e < R * nD; e += kGsThreads) fb[e] = dw_to_double(c.a.fb[e]);
    for (int i = c.tid; i < R; i += kGsThreads) p.coef[(size_t)iv * R + i] = dw_to_double(c.a.fcs[i]);
  }
  if (iv < p.nbloc - 1 && iv % c.NC == c.gr) {
    const int kl = iv / c.NC;
    dw* qf = c.a.qf + (size_t)kl * R * nD;
    dw* qw = c.a.qw + (size_t)kl * R * nD;
    for (int e = c.tid; e < R * nD; e += kGsThreads) {
      const dw x = c.a.fb[e];
      qf[e] = x;
      qw[e] = dw_mul(c.a.fcs[e / nD], x);
    }
    for (int i = c.tid; i < R; i += kGsThreads) c.a.qc[(size_t)kl * R + i] = c.a.fcs[i];
  }
  __syncthreads();
}

// Step phase 1.  Unless the previous step's update already formed them
// (`pre`), the products over d != j of the owned overlaps (psn) and of the
// working Grams (Gp, and BB = Gp + pen I).  Always: the weighted factor
// wf(r,m) = c_r F_r^j(m), and per warp of psn entries the partial sums of
// c_k,r c_i P_k(r,i) over all modes (the coefficients <Q_k, F>).
// Threads t0..511 (t0 a multiple of 32); ends with a barrier over them.
__device__ void step_products(const Gs& c, int j, int nk, bool pre, int t0, dw qinv) {
  const int R = c.R, RR = c.RR, RRp = c.RRp, D = c.D, nj = c.a.nb[j], offj = c.a.off[j];
  const int npsn = nk * RRp, ngp = npsn + (pre ? 0 : RR), total = ngp + R * nj;
  const dw pen = c.a.misc[0];
  for (int e = c.tid - t0; e < total; e += kGsThreads - t0) {
    if (e < npsn) {  // whole warps: npsn is a multiple of 32
      int kl, ee;
      c.a.fd[2].divmod((unsigned)e, &kl, &ee);
      dw contrib = dw_make(0.f);
      if (ee < RR) {
        int r, i;
        c.a.fd[0].divmod((unsigned)ee, &r, &i);
        const dw* Pk = c.a.P + (size_t)kl * D * RR + ee;
        const dw pj = Pk[(size_t)j * RR], w = dw_mul(c.a.qc[(size_t)kl * R + r], dw_mul(c.a.fcs[i], qinv));
        dw prod;
        if (pre) {
          prod = c.a.psn[(size_t)kl * RR + ee];
        } else {
          prod = dw_make(1.f);
          for (int d = 0; d < D; ++d)
            if (d != j) prod = dw_mul(prod, Pk[(size_t)d * RR]);
        }
        contrib = dw_mul(dw_mul(prod, pj), w);
        if (!pre) c.a.psn[(size_t)kl * RR + ee] = prod;
      }
      for (int o = 16; o > 0; o >>= 1) contrib = dw_add(contrib, dwsolve::dw_shfl_xor(contrib, o));
      if ((c.tid & 31) == 0) c.a.gpart[kl * (RRp / 32) + ee / 32] = contrib;
    } else if (e < ngp) {
      const int ee = e - npsn;
      dw prod = dw_make(1.f);
      for (int d = 0; d < D; ++d)
        if (d != j) prod = dw_mul(prod, c.a.g[(size_t)d * RR + ee]);
      c.a.Gp[ee] = prod;
      int i2, i;
      c.a.fd[0].divmod((unsigned)ee, &i2, &i);
      c.a.BB[ee] = mask_bb(c, i, i2, (i == i2) ? dw_add(prod, pen) : prod);
    } else {
      const int ee = e - ngp;
      int m, r;
      c.a.fd[0].divmod((unsigned)ee, &m, &r);
      c.a.wf[ee] = dw_mul(dw_mul(c.a.fcs[r], qinv), c.a.fb[(size_t)r * c.nD + offj + m]);
    }
  }
  if (t0 == 0) __syncthreads();
  else worker_sync(t0);
}

// Step phase 2 (threads w0..511, while the lower warps invert BB): the dot
// products over r, split in two halves,
//   source 0:        sum_r wf(r,m) Gp(r,i)                      (self term)
//   source 1 + kl:   sum_r c_k,r Q_k,r^j(m) psn_k(r,i)          (owned k)
// at part[(2 s + h) R nj + i + m R]; and gco_k = -<Q_k, F> from the partials.
__device__ void step_dots(const Gs& c, int j, int nk, int w0) {
  const int R = c.R, RR = c.RR, nj = c.a.nb[j], offj = c.a.off[j], Rn = R * nj, half = (R + 1) / 2;
  const int total = (nk + 1) * 2 * Rn, w = c.tid - w0, nw = kGsThreads - w0;
  const FastDiv fdrn = c.a.fd[3 + j];
  for (int e = w; e < total; e += nw) {
    int sh, em, m, i;
    fdrn.divmod((unsigned)e, &sh, &em);
    c.a.fd[0].divmod((unsigned)em, &m, &i);
    const int s = sh >> 1;
    const int r0 = (sh & 1) ? half : 0, r1 = (sh & 1) ? R : half;
    dw_acc acc = acc_zero();
    if (s == 0) {
      for (int r = r0; r < r1; ++r) acc_fma(acc, c.a.wf[r + m * R], c.a.Gp[r * R + i]);
    } else {
      const dw* A = c.a.qw + (size_t)(s - 1) * R * c.nD + offj + m;
      const dw* M = c.a.psn + (size_t)(s - 1) * RR + i;
      for (int r = r0; r < r1; ++r) acc_fma(acc, A[(size_t)r * c.nD], M[r * R]);
    }
    c.a.part[e] = acc_value(acc);
  }
  if (w < nk) {
    const int nch = c.RRp / 32;
    dw s = dw_make(0.f);
    for (int q = 0; q < nch; ++q) s = dw_add(s, c.a.gpart[w * nch + q]);
    c.a.gco[w] = dw_neg(s);
  }
  worker_sync(w0);
}

// Step phase 3 (threads w0..511): this CTA's part of the right-hand side,
//   sum_k gco_k sum_r c_k,r Q_k,r^j(m) psn_k(r,i).
__device__ void step_rhs_part(const Gs& c, int j, int nk, dw* bp, int w0) {
  const int Rn = c.R * c.a.nb[j];
  for (int e = c.tid - w0; e < Rn; e += kGsThreads - w0) {
    dw_acc acc = acc_zero();
    for (int kl = 0; kl < nk; ++kl) {
      const dw g = c.a.gco[kl];
      acc_fma(acc, g, c.a.part[(size_t)(2 * kl + 2) * Rn + e]);
      acc_fma(acc, g, c.a.part[(size_t)(2 * kl + 3) * Rn + e]);
    }
    bp[e] = acc_value(acc);
  }
}

// Step phase 4 (after the cluster barrier): the self term plus the partial
// right-hand sides of the cluster, summed as a fixed tree over ranks so that
// every CTA forms the identical system.  With several clusters (xout set)
// the cluster's sum alone goes to xout (by rank 0) and the grid-wide step
// below completes b0.
// (ranks >= nown own no earlier vector yet; their parts are exact zeros)
__device__ void step_gather(const Gs& c, int j, dw* bp, int nown, dw* xout = nullptr) {
  const int Rn = c.R * c.a.nb[j];
  for (int e = c.tid; e < Rn; e += kGsThreads) {
    const uint32_t local = (uint32_t)__cvta_generic_to_shared(bp + e);
    dw v[16];
#pragma unroll
    for (int r = 0; r < 16; ++r) {
      v[r] = dw_make(0.f);
      if (r < nown) {
        uint32_t remote;
        asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(r));
        asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v[r].hi), "=f"(v[r].lo) : "r"(remote) : "memory");
      }
    }
    dw_acc acc = acc_zero();
    if (xout) {
#pragma unroll
      for (int r = 0; r < 16; ++r) acc_add(acc, v[r]);
      if (c.rank == 0) xout[e] = acc_value(acc);
      continue;
    }
    acc_add(acc, c.a.part[e]);
    acc_add(acc, c.a.part[(size_t)Rn + e]);
#pragma unroll
    for (int r = 0; r < 16; ++r) acc_add(acc, v[r]);
    c.a.b0[e] = (e % c.R >= c.rv) ? dw_make(e / c.R == 0 ? 1.f : 0.f) : acc_value(acc);  // ragged padding
  }
  __syncthreads();
}

// Iterations of the bounded wait for the other clusters' partial sums (each
// a global load and a short sleep: about a tenth of a second in all, far
// above the imbalance of one mode step).
constexpr int kGridWaitLimit = 1 << 17;

// Grid-wide step (several clusters): once every cluster leader has posted
// its cluster sum for this step (xctr[0] >= G (step + 1)), every CTA forms
// b0 = self term + the cluster sums in cluster order -- the identical system
// everywhere.  The wait is bounded: the first CTA whose wait runs out sets
// status bit 2 and the abort word xctr[1], after which no CTA waits again;
// the kernel then runs to its end on whatever has arrived, and the result
// is flagged invalid.
__device__ void step_grid_sum(const Gs& c, const GsParams& p, int j, int step, const dw* xs) {
  const int Rn = c.R * c.a.nb[j];
  if (c.tid == 0) {
    if (c.rank == 0) {
      __threadfence();
      atomicAdd(p.xctr, 1u);
    }
    const unsigned target = (unsigned)c.G * (unsigned)(step + 1);
    volatile unsigned* ctr = p.xctr;
    for (int it = 0; ctr[0] < target && ctr[1] == 0u; ++it) {
      if (it >= kGridWaitLimit) {
        atomicExch(p.xctr + 1, 1u);
        atomicOr(p.status, 2);
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
  }
  __syncthreads();
  const size_t stride = (size_t)c.R * c.npm;
  for (int e = c.tid; e < Rn; e += kGsThreads) {
    dw_acc acc = acc_zero();
    acc_add(acc, c.a.part[e]);
    acc_add(acc, c.a.part[(size_t)Rn + e]);
    for (int g = 0; g < c.G; ++g) {
      const dw* x = xs + (size_t)g * stride + e;
      acc_add(acc, dw_make(__ldcg(&x->hi), __ldcg(&x->lo)));
    }
    c.a.b0[e] = (e % c.R >= c.rv) ? dw_make(e / c.R == 0 ? 1.f : 0.f) : acc_value(acc);  // ragged padding
  }
  __syncthreads();
}

// Step phase 5 (solver warps): X = BB^-1 b0 from the FP32 inverse formed
// during phases 2-4, rows normalised, norms as the new weights.
__device__ void step_solve(const Gs& c, int j, const float* inv, bool gj_ok) {
  const int R = c.R, nj = c.a.nb[j];
  int bad = 0;
  if (!(gj_ok && dwsolve::refine_solve(c.a.BB, R, c.a.b0, c.a.X, nj, inv, c.a.res, c.a.rred))) {
    for (int e = c.tid; e < R * nj; e += dwsolve::kSolverThreads) c.a.X[e] = c.a.b0[e];
    bad = dwsolve::dw_ldlt(c.a.BB, R, c.a.dinv, c.a.u);
    dwsolve::dw_ldlt_solve(c.a.BB, R, c.a.dinv, c.a.X, nj);
  }
  dwsolve::dw_normalise_rows(c.a.X, R, nj, c.a.fcs);
  if (c.tid == 0 && bad) c.a.flags[1] = 1;
}

// When another step of this vector follows (mode jn): the products over d
// not in {j, jn} of the owned overlaps (ppsn) and of the working Grams (pGp);
// the update multiplies in mode j.  Threads t0, t0 + nt, ...
__device__ void step_preproducts(const Gs& c, int j, int jn, int nk, int t0, int nt) {
  const int RR = c.RR, D = c.D;
  for (int e = t0; e < (nk + 1) * RR; e += nt) {
    int kl, ee;
    c.a.fd[1].divmod((unsigned)e, &kl, &ee);
    const bool own = kl < nk;
    const dw* src = own ? c.a.P + (size_t)kl * D * RR + ee : c.a.g + ee;
    dw prod = dw_make(1.f);
    for (int d = 0; d < D; ++d)
      if (d != j && d != jn) prod = dw_mul(prod, src[(size_t)d * RR]);
    if (own) c.a.ppsn[(size_t)kl * RR + ee] = prod;
    else c.a.pGp[ee] = prod;
  }
}

// Step phase 6: the new factor of mode j into the working vector, its Gram,
// and the owned overlaps of mode j; with `pre`, the next step's products
// psn, Gp and BB (mode jn) completed by multiplying in mode j.  Then the
// weights are divided by sqrt(<F,F>), whose terms c_i c_i' prod_d G_d(i,i')
// come with the new Gram.
__device__ dw step_update(const Gs& c, int j, int jn, int nk, bool pre) {
  const int R = c.R, RR = c.RR, nj = c.a.nb[j], offj = c.a.off[j], Rn = R * nj;
  const int total = Rn + RR + nk * RR;
  const dw pen = c.a.misc[0];
  dw qpart = dw_make(0.f);
  for (int e = c.tid; e < total; e += kGsThreads) {
    if (e < Rn) {
      int m, i;
      c.a.fd[0].divmod((unsigned)e, &m, &i);
      c.a.fb[(size_t)i * c.nD + offj + m] = c.a.X[e];
    } else if (e < Rn + RR) {
      const int ee = e - Rn;
      int i2, i;
      c.a.fd[0].divmod((unsigned)ee, &i2, &i);
      if (i > i2) continue;
      const int et = i2 + i * R;
      // prod_{d != j} G_d: Gp, or with `pre` pGp = prod_{d not in {j, jn}} G_d times G_jn
      const dw gp = pre ? c.a.pGp[ee] : c.a.Gp[ee], gq = pre ? dw_mul(gp, c.a.g[(size_t)jn * RR + ee]) : gp;
      const dw w = dw_mul(c.a.fcs[i], c.a.fcs[i2]);
      dw_acc acc = acc_zero();
      for (int m = 0; m < nj; ++m) acc_fma(acc, c.a.X[i + m * R], c.a.X[i2 + m * R]);
      const dw s = acc_value(acc);
      c.a.g[(size_t)j * RR + ee] = s;
      c.a.g[(size_t)j * RR + et] = s;
      dw t = dw_mul(dw_mul(gq, s), w);
      if (i != i2) t = dw{2.f * t.hi, 2.f * t.lo};
      qpart = dw_add(qpart, t);
      if (pre) {
        const dw gn = dw_mul(gp, s);
        c.a.Gp[ee] = gn;
        c.a.Gp[et] = gn;
        c.a.BB[ee] = mask_bb(c, i, i2, (i == i2) ? dw_add(gn, pen) : gn);
        c.a.BB[et] = c.a.BB[ee];
      }
    } else {
      int kl, e2, r, i;
      c.a.fd[1].divmod((unsigned)(e - Rn - RR), &kl, &e2);
      c.a.fd[0].divmod((unsigned)e2, &r, &i);
      const dw* x = c.a.qf + ((size_t)kl * R + r) * c.nD + offj;
      const dw pre_k = pre ? c.a.ppsn[(size_t)kl * RR + e2] : dw_make(1.f);
      dw_acc acc = acc_zero();
      for (int m = 0; m < nj; ++m) acc_fma(acc, x[m], c.a.X[i + m * R]);
      const dw s = acc_value(acc);
      c.a.P[((size_t)kl * c.D + j) * RR + e2] = s;
      if (pre) c.a.psn[(size_t)kl * RR + e2] = dw_mul(pre_k, s);
    }
  }
  // 1 / sqrt(<F,F>) for every thread: the next step's products apply it to
  // the weights as they read them (the solve then writes new weights), so
  // the weights need no rewrite and no barrier of their own here; the sum's
  // barrier also orders every write above before the next phase
  return dw_rcp(dw_sqrt(dw_abs(block_sum_ready(qpart, c.a.red))));
}

}  // namespace

// kResident: every array in shared memory (the compiler then addresses them
// as such); otherwise the groups of p.gmask live in global scratch.
template <bool kResident>
__global__ void __launch_bounds__(kGsThreads, 1) gs_kernel(GsParams p) {
  cg::cluster_group cluster = cg::this_cluster();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Gs c;
  c.CL = (int)cluster.num_blocks();
  c.rank = (int)cluster.block_rank();
  c.G = p.ngrp;
  c.cid = blockIdx.x / c.CL;
  c.gr = c.cid * c.CL + c.rank;
  c.NC = c.G * c.CL;
  c.R = p.R;
  c.RR = p.R * p.R;
  c.RRp = gs_rrp(p.R);
  c.D = p.D;
  c.nD = p.nD;
  c.npm = p.npmax;
  c.tid = threadIdx.x;
  c.rv = p.R;
  const GsDims dims{p.R, p.D, p.nD, p.npmax, p.nkmax, kResident ? 0 : p.gmask};
  gs_carve(dims, &c.a, smem_raw, reinterpret_cast<dw*>(p.work) + (size_t)c.gr * p.work_stride, nullptr);
  for (int d = c.tid; d <= c.D; d += kGsThreads) {
    c.a.nb[d] = d < c.D ? p.nbas[d] : 0;
    c.a.off[d] = p.off[d];
  }
  for (int q = c.tid; q < c.D + 3; q += kGsThreads)
    c.a.fd[q] = FastDiv((unsigned)(q == 0 ? c.R : q == 1 ? c.RR : q == 2 ? c.RRp : c.R * p.nbas[q - 3]));
  if (c.tid == 0) c.a.flags[1] = 0;
  __syncthreads();

  load_vector(c, p, 0);
  all_grams(c);
  normalize_weights(c);
  finish_vector(c, p, 0, false);

  int step = 0;
  for (int iv = 1; iv < p.nbloc && p.nals > 0; ++iv) {
    c.rv = p.rank_v ? p.rank_v[iv] : c.R;
    load_vector(c, p, iv);
    all_grams(c);
    const int nk = (iv - c.gr + c.NC - 1) / c.NC;  // owned k = gr, gr + NC, ... < iv
    all_overlaps(c, nk);
    bool pre = false;
    dw qinv = dw_make(1.f);  // 1 / |F| not yet applied to the weights (see step_update)
    for (int it = 0; it < p.nals; ++it) {
      for (int j = 0; j < c.D; ++j, ++step) {
        dw* bp = c.a.bpart + (size_t)(step & 1) * c.R * c.npm;
        const bool more = it + 1 < p.nals || j + 1 < c.D;  // another step of this vector follows
        const int jn = j + 1 < c.D ? j + 1 : 0, nj = c.a.nb[j];
        // FP32 inverse of BB (warp 0 in registers for R <= 32, else the
        // solver warps) concurrently with the right-hand side (threads w0..);
        // when the previous update already formed BB, also concurrently with
        // the products
        bool gj_ok = false;
        const float* inv = c.a.gi;
        const int w0 = c.R <= 32 ? 32 : dwsolve::kSolverThreads;
        const bool early = pre && c.R <= 32;
        if (!early) step_products(c, j, nk, pre, 0, qinv);
        if (c.tid < w0) {
          if (c.R > 32) {
            inv = dwsolve::gj_inverse(c.a.BB, c.R, c.a.gi, &gj_ok);
          } else {
            const bool good = dwsolve::gj_inverse_warp(c.a.BB, c.R, c.a.gi);
            if (c.tid == 0) c.a.flags[2] = good;
          }
        } else {
          if (early) step_products(c, j, nk, pre, w0, qinv);
          step_dots(c, j, nk, w0);
          step_rhs_part(c, j, nk, bp, w0);
        }
        // a peer's bpart of step s is rewritten at step s + 2, after every
        // CTA has passed the barrier of step s + 1 (and so its gather of s)
        cl_arrive();
        cl_wait();
        {
          // ranks of this cluster that own an earlier vector (the others' parts are zero)
          const int nown = min(c.CL, max(0, iv - c.cid * c.CL));
          if (c.G == 1) {
            step_gather(c, j, bp, nown);
          } else {
            dw* xs = p.xpart + (size_t)(step & 1) * c.G * c.R * c.npm;
            step_gather(c, j, bp, nown, xs + (size_t)c.cid * c.R * c.npm);
            step_grid_sum(c, p, j, step, xs);
          }
        }
        if (c.R <= 32) gj_ok = c.a.flags[2] != 0;
        // the solve: refinement in registers (warps 0..nsw-1, one or two
        // right-hand-side columns each), or the solver warps' refinement /
        // LDL^T fallback; the next step's partial products on the other warps
        bool solved = false, pre_done = !more;
        if (gj_ok && c.R <= 32 && nj <= 16) {
          // rank <= 16: one column per warp, sums split over the half-warps
          const bool split = c.R <= 16;
          const int nsw = (split ? nj : dwsolve::solve_cols_warps(c.R, nj)) * 32;
          if (c.tid < nsw) {
            const bool ok = split ? dwsolve::solve_cols_split(c.a.BB, c.R, c.a.b0, c.a.X, nj, inv, c.a.fcs, c.a.cs)
                                  : dwsolve::solve_cols_any(c.a.BB, c.R, c.a.b0, c.a.X, nj, inv, c.a.fcs, c.a.cs);
            if (c.tid == 0) c.a.flags[3] = ok;
          } else if (more) {
            step_preproducts(c, j, jn, nk, c.tid - nsw, kGsThreads - nsw);
          }
          __syncthreads();
          solved = c.a.flags[3] != 0;
          pre_done = pre_done || nsw < kGsThreads;
          gj_ok = false;  // not converged: straight to the LDL^T
        }
        if (!solved) {
          if (c.tid < dwsolve::kSolverThreads) step_solve(c, j, inv, gj_ok);
          else if (!pre_done) step_preproducts(c, j, jn, nk, c.tid - dwsolve::kSolverThreads, kWorkerThreads);
          __syncthreads();
          pre_done = true;
        }
        if (!pre_done) {
          step_preproducts(c, j, jn, nk, c.tid, kGsThreads);
          __syncthreads();
        }
        if (c.rv < c.R) {  // ragged: the padded terms keep zero weight
          for (int i = c.rv + c.tid; i < c.R; i += kGsThreads) c.a.fcs[i] = dw_make(0.f);
          __syncthreads();
        }
        qinv = step_update(c, j, jn, nk, more);
        pre = more;
      }
    }
    for (int i = c.tid; i < c.R; i += kGsThreads) c.a.fcs[i] = dw_mul(c.a.fcs[i], qinv);
    __syncthreads();
    finish_vector(c, p, iv, true);
  }
  if (c.gr == 0 && c.tid == 0 && c.a.flags[1]) atomicOr(p.status, 1);
  // no CTA leaves while a peer may still read its shared memory
  cl_arrive();
  cl_wait();
}

// CTAs per cluster: 16 (the non-portable maximum) unless the block is
// smaller or the caller asks for `pref` (the measured choice of
// gs_tuned_cluster); MLCP_GB300_GS_CLUSTER fixes a size (measurements).
int gs_cluster_size(int nbloc, int pref) {
  int cl = pref > 0 ? std::max(2, std::min(16, pref)) : 16;
  if (const char* e = getenv("MLCP_GB300_GS_CLUSTER")) cl = std::max(2, std::min(16, atoi(e)));
  return nbloc > cl ? cl : (nbloc > 1 ? nbloc - 1 : 1);
}

namespace {

// Most clusters a grid may hold (the GB300's 152 SMs at one 16-CTA cluster
// per 16 SMs); the scratch is sized for it.
constexpr int kMaxGroups = 9;

// Cluster sizes the search tries (each clamped to the block).
constexpr int kClusterCandidates[] = {16, 12, 8};

int gs_nkmax(int nbloc, int ngrp, int cl) {
  const int nc = gs_cluster_size(nbloc, cl) * ngrp;
  return std::max(1, (nbloc - 1 + nc - 1) / nc);
}

// Global scratch entries (dw) of one CTA with every movable group there.
size_t gs_cta_work(int nbloc, int R, int nD, int D, int npm, int ngrp, int cl) {
  GsArrays a;
  size_t gw = 0;
  gs_carve(GsDims{R, D, nD, npm, gs_nkmax(nbloc, ngrp, cl), kGroupAll}, &a, nullptr, nullptr, &gw);
  return gw;
}

// Shared-memory layout: keep as much resident as fits (the owned vectors
// move out first, then their overlaps, then the working vector).
bool gs_fit(const GsParams& p, int ngrp, int smem_max, int* gmask, size_t* smem) {
  static const int masks[4] = {0, kGroupQ, kGroupQ | kGroupP, kGroupAll};
  for (int q = 0; q < 4; ++q) {
    GsArrays a;
    const size_t b = gs_carve(GsDims{p.R, p.D, p.nD, p.npmax, gs_nkmax(p.nbloc, ngrp, p.cl), masks[q]}, &a,
                              nullptr, nullptr, nullptr);
    if (b <= (size_t)smem_max) {
      *gmask = masks[q];
      *smem = b;
      return true;
    }
  }
  return false;
}

}  // namespace

size_t gs_work_doubles(int nbloc, int R, int nD, int D, int npm) {
  // the per-CTA scratch of the largest grid (one cluster owns the most per
  // CTA, so size the scratch for every CTA of kMaxGroups clusters at the
  // one-cluster share), for every cluster size the search may pick, then
  // the cluster partials and the arrival counter
  size_t most = 0;
  for (int c : kClusterCandidates) {
    const int cl = gs_cluster_size(nbloc, c);
    most = std::max(most, (size_t)cl * kMaxGroups * gs_cta_work(nbloc, R, nD, D, npm, 1, c));
  }
  return most + (size_t)2 * kMaxGroups * R * npm + 2;
}

namespace {

// Clusters for a block: one when everything fits in shared memory (small
// blocks are bound by the latency of each mode step, and a grid-wide step
// would only add to it); otherwise as many as the SMs hold at one CTA each,
// up to one owned vector per CTA, so that the owned arrays' work spreads
// over more SMs.
int gs_groups(const GsParams& p, int num_sms, int smem_max) {
  int gmask = 0;
  size_t smem = 0;
  if (gs_fit(p, 1, smem_max, &gmask, &smem) && gmask == 0) return 1;
  const int cl = gs_cluster_size(p.nbloc, p.cl);
  int g = std::min(kMaxGroups, num_sms / cl);
  g = std::min(g, (p.nbloc - 1 + cl - 1) / cl);
  return std::max(1, g);
}

}  // namespace

int gs_launch(const GsParams& prm, cudaStream_t st) {
  GsParams p = prm;
  const int cl = gs_cluster_size(p.nbloc, p.cl);
  int dev = 0, smem_max = 0, nsm = 0;
  MLCP_CUDA_TRY(cudaGetDevice(&dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const char* env = getenv("MLCP_GB300_GS_GROUPS");  // a fixed cluster count (tests)
  int ngrp = env ? std::max(1, std::min(kMaxGroups, atoi(env))) : gs_groups(p, nsm, smem_max);
  if (ngrp * cl > nsm) ngrp = std::max(1, nsm / cl);
  void (*kern)(GsParams) = nullptr;
  size_t smem = 0;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[2];
  for (int pass = 0;; ++pass) {
    p.ngrp = ngrp;
    p.nkmax = gs_nkmax(p.nbloc, ngrp, p.cl);
    p.work_stride = (long long)gs_cta_work(p.nbloc, p.R, p.nD, p.D, p.npmax, ngrp, p.cl);
    int gmask = 0;
    if (!gs_fit(p, ngrp, smem_max, &gmask, &smem)) {
      set_error("intertwinecpp_: Gram-Schmidt needs more shared memory than %d bytes (rank %d)", smem_max, p.R);
      return kTooLarge;
    }
    p.gmask = gmask;
    kern = p.gmask == 0 ? gs_kernel<true> : gs_kernel<false>;
    MLCP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (cl > 8) MLCP_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cfg = {};
    cfg.gridDim = dim3(cl * ngrp);
    cfg.blockDim = dim3(kGsThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cl;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    // several clusters wait on one another each step: all of them must be
    // resident together, which a cooperative launch guarantees (or refuses)
    attr[1].id = cudaLaunchAttributeCooperative;
    attr[1].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (ngrp == 1) break;
    // no more clusters than the GPU holds at once at this size and shared
    // memory (the GPCs bound how many clusters of 8-16 CTAs fit); with fewer
    // clusters each CTA owns more earlier vectors, so the layout is redone
    int maxc = 0;
    MLCP_CUDA_TRY(cudaOccupancyMaxActiveClusters(&maxc, (const void*)kern, &cfg));
    if (maxc >= ngrp || pass >= 3) break;
    ngrp = std::max(1, maxc);
  }
  // the cluster partials and the arrival counter follow the per-CTA scratch
  dw* after = reinterpret_cast<dw*>(p.work) + (size_t)cl * ngrp * p.work_stride;
  p.xpart = after;
  p.xctr = reinterpret_cast<unsigned*>(after + (size_t)2 * kMaxGroups * p.R * p.npmax);
  if (ngrp > 1) MLCP_CUDA_TRY(cudaMemsetAsync(p.xctr, 0, 2 * sizeof(unsigned), st));  // arrivals, abort word
  cfg.numAttrs = ngrp > 1 ? 2 : 1;
  MLCP_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, p));
  return kOk;
}

// ---------------------------------------------------------------------------
// Cluster-size search
// ---------------------------------------------------------------------------
// A larger cluster spreads the earlier vectors over more CTAs but pays a
// longer gather and cluster barrier at every mode step; which wins depends on
// the block (measured on the 40-vector rank-16 block: 16 CTAs 27.7 ms per
// cycle, 12 CTAs 28.7, 8 CTAs 31.2).  The first cycle of a block shape runs
// one Gram-Schmidt sweep (nals = 1) twice with each candidate size on a
// scratch copy of the block, times it with CUDA events on the cycle's stream
// and caches the size of the fastest run for the process, per device and
// shape.  Off with
// mlcp_gb300_set_autotune(0) / MLCP_GB300_AUTOTUNE=0 or a fixed
// MLCP_GB300_GS_CLUSTER (then the 16-CTA rule applies).

namespace {

struct GsTuneKey {
  int device, nbloc, R, D, nD, npmax, ragged;
  bool operator<(const GsTuneKey& o) const {
    return std::tie(device, nbloc, R, D, nD, npmax, ragged) <
           std::tie(o.device, o.nbloc, o.R, o.D, o.nD, o.npmax, o.ragged);
  }
};

struct GsTuneEntry {
  int cl = 0;
  std::vector<std::pair<int, float>> trials;  // (cluster size, ms of one sweep)
};

std::mutex g_gs_tune_mu;
std::map<GsTuneKey, GsTuneEntry> g_gs_tune;

}  // namespace

int gs_tuned_cluster(const GsParams& p, int device, double* scratch_base, double* scratch_coef, cudaStream_t st,
                     int* cl_out) {
  *cl_out = 0;
  if (getenv("MLCP_GB300_GS_CLUSTER") || p.nals <= 0) return kOk;
  const GsTuneKey key{device, p.nbloc, p.R, p.D, p.nD, p.npmax, p.rank_v != nullptr};
  {
    std::lock_guard<std::mutex> lk(g_gs_tune_mu);
    auto it = g_gs_tune.find(key);
    if (it != g_gs_tune.end()) {
      *cl_out = it->second.cl;
      return kOk;
    }
  }
  std::vector<int> cand;
  for (int c : kClusterCandidates) {
    const int cl = gs_cluster_size(p.nbloc, c);
    if (std::find(cand.begin(), cand.end(), cl) == cand.end()) cand.push_back(cl);
  }
  GsTuneEntry entry;
  if (cand.size() > 1) {
    const size_t nvals = (size_t)p.nbloc * p.R * p.nD, ncoef = (size_t)p.nbloc * p.R;
    cudaEvent_t e0, e1;
    MLCP_CUDA_TRY(cudaEventCreate(&e0));
    MLCP_CUDA_TRY(cudaEventCreate(&e1));
    float best = 0.f;
    for (int cl : cand) {
      GsParams t = p;
      t.base = scratch_base;
      t.coef = scratch_coef;
      t.nals = 1;
      t.cl = cl;
      float ms = -1.f;
      for (int rep = 0; rep < 2; ++rep) {  // the faster of two runs
        MLCP_CUDA_TRY(cudaMemcpyAsync(scratch_base, p.base, sizeof(double) * nvals, cudaMemcpyDeviceToDevice, st));
        MLCP_CUDA_TRY(cudaMemcpyAsync(scratch_coef, p.coef, sizeof(double) * ncoef, cudaMemcpyDeviceToDevice, st));
        MLCP_CUDA_TRY(cudaEventRecord(e0, st));
        if (gs_launch(t, st) != kOk) {  // a size this GPU cannot launch for the block: no candidate
          cudaGetLastError();
          ms = -1.f;
          break;
        }
        MLCP_CUDA_TRY(cudaEventRecord(e1, st));
        MLCP_CUDA_TRY(cudaEventSynchronize(e1));
        float m = 0.f;
        MLCP_CUDA_TRY(cudaEventElapsedTime(&m, e0, e1));
        ms = (ms < 0.f || m < ms) ? m : ms;
      }
      if (ms < 0.f) continue;
      entry.trials.push_back({cl, ms});
      if (entry.trials.size() == 1 || ms < best) {
        best = ms;
        entry.cl = cl;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  } else {
    entry.cl = cand.empty() ? 0 : cand[0];
  }
  {
    std::lock_guard<std::mutex> lk(g_gs_tune_mu);
    g_gs_tune[key] = entry;
  }
  *cl_out = entry.cl;
  return kOk;
}

void gs_tune_report(std::string& out) {
  std::lock_guard<std::mutex> lk(g_gs_tune_mu);
  char line[160];
  for (const auto& kv : g_gs_tune) {
    const GsTuneKey& k = kv.first;
    snprintf(line, sizeof(line), "gs nbloc=%d R=%d ndof=%d nD=%d%s: cluster %d;", k.nbloc, k.R, k.D, k.nD,
             k.ragged ? " ragged" : "", kv.second.cl);
    out += line;
    for (const auto& t : kv.second.trials) {
      snprintf(line, sizeof(line), " %d=%.3fms", t.first, t.second);
      out += line;
    }
    out += "\n";
  }
}

}  // namespace mlcp
