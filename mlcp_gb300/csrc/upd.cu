// Vector updates of the intertwined cycle in double-word arithmetic.
//
// Reference: VectorUpdates / UPDATES_ALS (src/intertw_lcv.cu:209-304) with
// lcv_build_linear_system(gs = false) (:75-127).  Every vector i of the block
// is replaced by the rank-R ALS fit, started from Q_i itself, of the linear
// combination sum_k U(k,i) Q_k of the block's old vectors (U: the
// eigenvectors of the Rayleigh-Ritz problem), nals sweeps over the modes,
// then its weights are divided by its norm.  Mode step k:
//   b(i',n)   = sum_{l,r} U(l,i) c_{l,r} Q_{l,r}^k(n) prod_{d!=k} <Q_{l,r}^d, F_i'^d>
//   BB(i',i") = prod_{d!=k} <F_i'^d, F_i"^d> + pen delta,  pen = 1e-10 max c(Q_i)
//   F^k = rows of BB^-1 b, normalised (the norms become the weights).
// The penalty is the reference's FP64-build rule (src/als.cu:248-267): a
// nearly converged block makes these normal equations ill-conditioned up to
// the penalty, so b is formed in double-word arithmetic (about 48 bits), as
// are the Grams and the solve; FP32 right-hand sides are not accurate enough
// for that rule.
//
// GB300 layout: a cluster of cl CTAs per output vector (the updates are
// independent: the reference writes each new vector to the host and keeps
// fitting the old block); cl is the largest of 1-4 that keeps the whole
// block's clusters on the SMs at once.  The block's factors are converted
// once to a double-word, mode-major copy shared by all CTAs (the mode-k
// slice of all B R terms is one contiguous run, L2-resident).  CTA `rank`
// of a cluster owns a contiguous range of the B R block terms lr and keeps
// the per-mode overlaps Gram_d(i', lr) = <Q_lr^d, F_i'^d> of its terms with
// the fitted vector's terms i' (only mode k changes per step), in shared
// memory when they fit, else in global scratch; every CTA keeps the same F
// Grams.  The right-hand side streams the CTA's block terms through shared
// memory in tiles: the products w_lr prod_{d!=k} Gram_d(i', lr) of a tile
// first, then the contraction with the tile's mode-k factors, while warp 0
// inverts BB in registers (the refinement's preconditioner).  The partial
// right-hand sides meet through distributed shared memory, summed in rank
// order, so every CTA solves the identical system and holds the identical
// new factor; one cluster barrier per mode step.
#include <cooperative_groups.h>

#include <algorithm>

#include "common.cuh"
#include "dword.cuh"
#include "dwsolve.cuh"
#include "intertwine.cuh"

namespace cg = cooperative_groups;

namespace mlcp {

namespace {

constexpr int kThreads = 512;
constexpr int kMaxCl = 4;
constexpr int kWarps = kThreads / 32;

struct UpdSmem {
  dw* X;      // [R][npmax] solution (column-major, ld R)
  dw* b0;     // [R][npmax] right-hand side
  dw* res;    // [R][npmax] refinement residual
  dw* BB;     // [R][R]
  float* gi;  // [2][R][R] FP32 inverse of BB
  dw* cf;     // [R] weights of F (row norms)
  dw* dinv;   // [R]
  dw* u;      // [R]
  dw* misc;   // [2] penalty, norm
  dw* red;    // [kWarps]
  float* rred;
  dwsolve::ColScratch cs;
  dw* P;      // [R][TL] products of one tile of block terms
  dw* Qt;     // [TL][npmax] mode-k factors of the tile
  dw* bacc;   // [max(nw, R*npmax)] partial right-hand sides
  dw* bpart;  // [2][R*npmax] this CTA's partial right-hand side (read by the cluster)
  dw* gram;   // [D][R][nlr] block overlaps of the CTA's terms (resident form only)
  int* flags; // [4]
};

// Shared memory; D and nlr (block terms per CTA) only matter for the resident form.
__host__ __device__ inline size_t upd_carve(UpdSmem& s, unsigned char* base, int R, int npm, int TL, int D = 0,
                                            int nlr = 0, bool resident = false) {
  size_t o = 0;
  auto take = [&](size_t bytes) -> unsigned char* {
    const size_t r = o;
    o += (bytes + 15) / 16 * 16;
    return base ? base + r : nullptr;
  };
  const size_t Rn = (size_t)R * npm, RR = (size_t)R * R;
  s.X = (dw*)take(sizeof(dw) * Rn);
  s.b0 = (dw*)take(sizeof(dw) * Rn);
  s.res = (dw*)take(sizeof(dw) * Rn);
  s.BB = (dw*)take(sizeof(dw) * RR);
  s.gi = (float*)take(sizeof(float) * 2 * RR);
  s.cf = (dw*)take(sizeof(dw) * R);
  s.dinv = (dw*)take(sizeof(dw) * R);
  s.u = (dw*)take(sizeof(dw) * R);
  s.misc = (dw*)take(sizeof(dw) * 2);
  s.red = (dw*)take(sizeof(dw) * kWarps);
  s.rred = (float*)take(sizeof(float) * 4);
  s.cs.conv = (float*)take(sizeof(float) * 64);
  s.cs.rmax = (float*)take(sizeof(float) * 16 * 32);
  s.cs.rsum = (dw*)take(sizeof(dw) * 16 * 32);
  s.P = (dw*)take(sizeof(dw) * (size_t)R * TL);
  s.Qt = (dw*)take(sizeof(dw) * (size_t)TL * npm);
  s.bacc = (dw*)take(sizeof(dw) * (Rn > (size_t)kThreads ? Rn : (size_t)kThreads));
  s.bpart = (dw*)take(sizeof(dw) * 2 * Rn);
  s.gram = resident ? (dw*)take(sizeof(dw) * (size_t)D * R * nlr) : nullptr;
  s.flags = (int*)take(sizeof(int) * 4);
  return o;
}

__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// Block terms per CTA when cl CTAs share a vector's B R terms.
__host__ __device__ inline int upd_per(int BR, int cl) { return (BR + cl - 1) / cl; }

// Global scratch (dw) of one CTA: overlaps (non-resident form), F Grams, target weights.
__host__ __device__ inline size_t upd_cta_dw(int BR, int R, int D, int cl) {
  const size_t per = (size_t)upd_per(BR, cl);
  return (size_t)D * R * per + (size_t)D * R * R + per;
}

// Block factors to the double-word mode-major copy: mode d of block term lr
// at qdw[off[d] * BR + lr * n_d + m].
__global__ void upd_prep_kernel(UpdParams p) {
  const int BR = p.B * p.R;
  const long long n = (long long)BR * p.nD;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
       e += (long long)gridDim.x * blockDim.x) {
    const int lr = (int)(e / p.nD), c = (int)(e - (long long)lr * p.nD);
    int d = 0;
    while (p.off[d + 1] <= c) ++d;
    const int m = c - p.off[d], nd = p.off[d + 1] - p.off[d];
    p.qdw[(size_t)p.off[d] * BR + (size_t)lr * nd + m] = dw_from_double(p.q[e]);
  }
}

__device__ dw block_sum(dw v, dw* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v = dw_add(v, dwsolve::dw_shfl_xor(v, o));
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  dw s = dw_make(0.f);
  if (threadIdx.x == 0)
    for (int w = 0; w < kWarps; ++w) s = dw_add(s, red[w]);
  return s;
}

__global__ void __launch_bounds__(kThreads, 1) upd_kernel(UpdParams p) {
  cg::cluster_group cluster = cg::this_cluster();
  const int CL = p.cl, rank = CL > 1 ? (int)cluster.block_rank() : 0;
  const int i = blockIdx.x / CL;
  const int R = p.R, B = p.B, D = p.D, nD = p.nD, npm = p.npmax, RR = R * R, BR = B * R, TL = p.tile;
  const int per = upd_per(BR, CL), lr0 = min(BR, rank * per), nlr = min(BR, lr0 + per) - lr0;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  UpdSmem s;
  upd_carve(s, smem_raw, R, npm, TL, D, per, p.resident != 0);
  dw* scr = p.work + (size_t)(i * CL + rank) * upd_cta_dw(BR, R, D, CL);
  dw* gram = p.resident ? s.gram : scr;          // [D][R][nlr]: <Q_lr^d, F_i'^d>, own terms lr0.., lr fastest
  dw* fg = scr + (size_t)D * R * per;            // [D][R][R] F Grams (the same in every CTA of the cluster)
  dw* w = fg + (size_t)D * RR;                   // [nlr] target weights U(l,i) c_lr of the own terms
  double* fb = p.qn + (size_t)i * R * nD;
  double* fc = p.qnc + (size_t)i * R;
  const double* qi = p.q + (size_t)i * R * nD;

  // ---- set-up: F = Q_i, target weights, penalty, Grams ----
  if (rank == 0)
    for (int e = threadIdx.x; e < R * nD; e += kThreads) fb[e] = qi[e];
  for (int c = threadIdx.x; c < nlr; c += kThreads) {
    const int lr = lr0 + c;
    w[c] = dw_from_double(p.U[lr / R + (size_t)i * B] * p.qc[lr]);
  }
  if (threadIdx.x == 0) {
    double pen = p.qc[(size_t)i * R];
    for (int r = 1; r < R; ++r) pen = p.qc[(size_t)i * R + r] > pen ? p.qc[(size_t)i * R + r] : pen;
    s.misc[0] = dw_from_double(pen * p.pen_factor);
    s.flags[1] = 0;
  }
  for (int d = 0; d < D; ++d) {
    const int nd = p.nbas[d], od = p.off[d];
    const dw* qd = p.qdw + (size_t)od * BR;
    const dw* fd = p.qdw + (size_t)od * BR + (size_t)i * R * nd;  // F = Q_i: its own terms in the copy
    for (int e = threadIdx.x; e < R * nlr; e += kThreads) {
      const int ip = e / nlr, c = e - ip * nlr;
      dw_acc acc = acc_zero();
      for (int m = 0; m < nd; ++m) acc_fma(acc, qd[(size_t)(lr0 + c) * nd + m], fd[(size_t)ip * nd + m]);
      gram[(size_t)d * R * nlr + e] = acc_value(acc);
    }
    for (int e = threadIdx.x; e < RR; e += kThreads) {
      const int a = e % R, c = e / R;
      dw_acc acc = acc_zero();
      for (int m = 0; m < nd; ++m) acc_fma(acc, fd[(size_t)a * nd + m], fd[(size_t)c * nd + m]);
      fg[(size_t)d * RR + e] = acc_value(acc);
    }
  }
  __syncthreads();
  const dw pen = s.misc[0];
  const int rv = p.rank_v ? p.rank_v[i] : R;  // ragged: this vector's rank

  int step = 0;
  for (int sw = 0; sw < p.nals; ++sw) {
    for (int k = 0; k < D; ++k, ++step) {
      const int nk = p.nbas[k], ok = p.off[k];
      const dw* qk = p.qdw + (size_t)ok * BR;
      dw* bp = s.bpart + (size_t)(step & 1) * R * npm;
      // -- normal equations --
      for (int e = threadIdx.x; e < RR; e += kThreads) {
        dw bb = dw_make(1.f);
        for (int d = 0; d < D; ++d)
          if (d != k) bb = dw_mul(bb, fg[(size_t)d * RR + e]);
        if (e % R == e / R) bb = dw_add(bb, pen);
        if (e % R >= rv || e / R >= rv) bb = dw_make(e % R == e / R ? 1.f : 0.f);  // ragged: decoupled padding
        s.BB[e] = bb;
      }
      __syncthreads();
      const int w0 = R <= 32 ? 32 : dwsolve::kSolverThreads;
      if (threadIdx.x < w0) {
        if (R <= 32) {
          const bool g = dwsolve::gj_inverse_warp(s.BB, R, s.gi);
          if (threadIdx.x == 0) {
            s.flags[2] = g;
            s.flags[0] = 0;
          }
        } else {
          bool ok2;
          const float* iv = dwsolve::gj_inverse(s.BB, R, s.gi, &ok2);
          if (threadIdx.x == 0) {
            s.flags[2] = ok2;
            s.flags[0] = iv == s.gi ? 0 : 1;
          }
        }
      } else {
        // -- this CTA's part of the right-hand side, tile by tile over its block terms --
        const int wt = threadIdx.x - w0, nw = kThreads - w0;
        const int nout = R * nk;
        const int nsl = nout >= nw ? 1 : nw / nout;  // slices of a tile per output
        const int items = nout * nsl;
        for (int it = wt; it < items; it += nw) s.bacc[it] = dw_make(0.f);
        for (int c0 = 0; c0 < nlr; c0 += TL) {
          const int tl = min(TL, nlr - c0);
          for (int e = wt; e < R * tl; e += nw) {
            const int ip = e / tl, c = e - ip * tl;
            dw pr = w[c0 + c];
            for (int d = 0; d < D; ++d)
              if (d != k) pr = dw_mul(pr, gram[(size_t)d * R * nlr + (size_t)ip * nlr + c0 + c]);
            s.P[ip * TL + c] = pr;
          }
          for (int e = wt; e < tl * nk; e += nw) s.Qt[e] = qk[(size_t)(lr0 + c0) * nk + e];
          asm volatile("bar.sync 2, %0;" ::"r"(nw) : "memory");
          for (int it = wt; it < items; it += nw) {
            const int o = it % nout, sl = it / nout;
            const int ip = o % R, m = o / R;
            const int a0 = sl * tl / nsl, a1 = (sl + 1) * tl / nsl;
            dw_acc acc = acc_zero();
            for (int c = a0; c < a1; ++c) acc_fma(acc, s.P[ip * TL + c], s.Qt[c * nk + m]);
            s.bacc[it] = dw_add(s.bacc[it], acc_value(acc));
          }
          asm volatile("bar.sync 2, %0;" ::"r"(nw) : "memory");
        }
        for (int o = wt; o < nout; o += nw) {
          dw b = s.bacc[o];
          for (int sl = 1; sl < nsl; ++sl) b = dw_add(b, s.bacc[sl * nout + o]);
          const int ip = o % R, m = o / R;
          bp[ip + m * R] = b;
        }
      }
      // -- the cluster's partial right-hand sides, summed in rank order (a
      // peer's part of step s is rewritten at step s + 2, after every CTA has
      // passed the barrier of step s + 1 and so finished its gather of s) --
      if (CL > 1) {
        cl_arrive();
        cl_wait();
      } else {
        __syncthreads();
      }
      for (int e = threadIdx.x; e < R * nk; e += kThreads) {
        const int ip = e % R, m = e / R;
        dw b;
        if (CL > 1) {
          const uint32_t local = (uint32_t)__cvta_generic_to_shared(bp + e);
          dw v[kMaxCl];
#pragma unroll
          for (int r = 0; r < kMaxCl; ++r) {
            v[r] = dw_make(0.f);
            if (r < CL) {
              uint32_t remote;
              asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(r));
              asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v[r].hi), "=f"(v[r].lo) : "r"(remote)
                           : "memory");
            }
          }
          b = v[0];
#pragma unroll
          for (int r = 1; r < kMaxCl; ++r)
            if (r < CL) b = dw_add(b, v[r]);
        } else {
          b = bp[e];
        }
        s.b0[e] = ip >= rv ? dw_make(m == 0 ? 1.f : 0.f) : b;
      }
      __syncthreads();
      // -- solve (as in the power sweep) --
      bool gj_ok = s.flags[2] != 0;
      const float* inv = s.gi + (size_t)s.flags[0] * RR;
      bool solved = false;
      const int nsw = dwsolve::solve_cols_warps(R, nk);
      if (gj_ok && R <= 32 && nk <= 16 && nsw <= kWarps) {
        if (threadIdx.x < nsw * 32) {
          const bool ok2 = dwsolve::solve_cols_any(s.BB, R, s.b0, s.X, nk, inv, s.cf, s.cs);
          if (threadIdx.x == 0) s.flags[3] = ok2;
        }
        __syncthreads();
        solved = s.flags[3] != 0;
        gj_ok = false;
      }
      if (!solved) {
        if (threadIdx.x < dwsolve::kSolverThreads) {
          int bad = 0;
          if (!(gj_ok && dwsolve::refine_solve(s.BB, R, s.b0, s.X, nk, inv, s.res, s.rred))) {
            for (int e = threadIdx.x; e < R * nk; e += dwsolve::kSolverThreads) s.X[e] = s.b0[e];
            bad = dwsolve::dw_ldlt(s.BB, R, s.dinv, s.u);
            dwsolve::dw_ldlt_solve(s.BB, R, s.dinv, s.X, nk);
          }
          dwsolve::dw_normalise_rows(s.X, R, nk, s.cf);
          if (threadIdx.x == 0 && bad) s.flags[1] = 1;
        }
        __syncthreads();
      }
      for (int r = rv + threadIdx.x; r < R; r += kThreads) s.cf[r] = dw_make(0.f);  // ragged: weightless padding
      // -- the new factor: FP64 output (rank 0), its Gram, the own block overlaps of mode k --
      if (rank == 0)
        for (int e = threadIdx.x; e < R * nk; e += kThreads) {
          const int ip = e / nk, m = e % nk;
          fb[(size_t)ip * nD + ok + m] = dw_to_double(s.X[ip + m * R]);
        }
      for (int e = threadIdx.x; e < RR; e += kThreads) {
        const int a = e % R, c = e / R;
        if (a > c) continue;
        dw_acc acc = acc_zero();
        for (int m = 0; m < nk; ++m) acc_fma(acc, s.X[a + m * R], s.X[c + m * R]);
        const dw g = acc_value(acc);
        fg[(size_t)k * RR + a + c * R] = g;
        fg[(size_t)k * RR + c + a * R] = g;
      }
      for (int e = threadIdx.x; e < R * nlr; e += kThreads) {
        const int ip = e / nlr, c = e - ip * nlr;
        dw_acc acc = acc_zero();
        for (int m = 0; m < nk; ++m) acc_fma(acc, qk[(size_t)(lr0 + c) * nk + m], s.X[ip + m * R]);
        gram[(size_t)k * R * nlr + e] = acc_value(acc);
      }
      __syncthreads();
    }
  }
  // ---- weights divided by the norm (src/intertw_lcv.cu:269-273) ----
  if (p.nals > 0) {
    dw part = dw_make(0.f);
    for (int e = threadIdx.x; e < RR; e += kThreads) {
      dw prod = dw_mul(s.cf[e % R], s.cf[e / R]);
      for (int d = 0; d < D; ++d) prod = dw_mul(prod, fg[(size_t)d * RR + e]);
      part = dw_add(part, prod);
    }
    const dw tot = block_sum(part, s.red);
    if (threadIdx.x == 0) s.misc[1] = dw_sqrt(dw_abs(tot));
    __syncthreads();
    const dw q = s.misc[1];
    if (rank == 0)
      for (int r = threadIdx.x; r < R; r += kThreads) fc[r] = dw_to_double(dw_div(s.cf[r], q));
  } else if (rank == 0) {
    for (int r = threadIdx.x; r < R; r += kThreads) fc[r] = p.qc[(size_t)i * R + r];
  }
  if (threadIdx.x == 0 && rank == 0 && s.flags[1]) atomicOr(&p.status[i], 1);
  // no CTA leaves while a peer may still read its shared memory
  if (CL > 1) {
    cl_arrive();
    cl_wait();
  }
}

}  // namespace

size_t upd_work_dw(int B, int R, int D) {
  size_t most = 0;
  for (int cl = 1; cl <= kMaxCl; ++cl) most = std::max(most, (size_t)B * cl * upd_cta_dw(B * R, R, D, cl));
  return most;
}

size_t upd_qdw_dw(int B, int R, int nD) { return (size_t)B * R * nD; }

int upd_launch(UpdParams p, int smem_optin, cudaStream_t st) {
  int dev = 0, nsm = 0;
  MLCP_CUDA_TRY(cudaGetDevice(&dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  // CTAs per vector: the most (up to 4) that keeps every cluster of the block
  // on the SMs at once; the block overlaps resident when they fit
  int cl = kMaxCl;
  while (cl > 1 && p.B * cl > nsm) --cl;
  const int BR = p.B * p.R, per = upd_per(BR, cl);
  int tile = 0, resident = 0;
  size_t smem = 0;
  for (int res = 1; res >= 0 && !tile; --res)
    for (int tl = 128; tl >= 16; tl /= 2) {
      UpdSmem s;
      smem = upd_carve(s, nullptr, p.R, p.npmax, tl, p.D, per, res != 0);
      if (smem <= (size_t)smem_optin) {
        tile = tl;
        resident = res;
        break;
      }
    }
  if (!tile) {
    set_error("vector updates: rank %d with %d basis functions needs more shared memory than %d bytes", p.R,
              p.npmax, smem_optin);
    return kTooLarge;
  }
  p.tile = tile;
  p.cl = cl;
  p.resident = resident;
  const long long n = (long long)p.B * p.R * p.nD;
  upd_prep_kernel<<<(int)std::min<long long>((n + 255) / 256, 4096), 256, 0, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  MLCP_CUDA_TRY(cudaFuncSetAttribute(upd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p.B * cl);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MLCP_CUDA_TRY(cudaLaunchKernelEx(&cfg, upd_kernel, p));
  return kOk;
}

}  // namespace mlcp
