// ALS-guided Gram-Schmidt over a block of CP vectors (reference GramSchmidt,
// src/intertw_lcv.cu:131-205, with lcv_build_linear_system :77-127).
//
// Vector iv (iv >= 1) is fitted, mode by mode, to
//   F - sum_{k<iv} <Q_k, F> Q_k,
// where F is its current iterate and the coefficients <Q_k, F> are
// recomputed at every mode step (gramsumoverrow + sumarray in the reference).
// The pairwise per-mode overlaps P(k,d) = Q_{k,d} F_d^T (R x R) are kept and
// only the mode just solved is refreshed, so a mode step costs
// O(iv R^2 (D + 2n)) instead of rebuilding every product over all modes.
// Everything here runs in FP64: once power iteration has made the block's
// vectors nearly parallel, the target F - sum_k <Q_k,F> Q_k is a small
// difference of large terms, and FP32 contractions lose it to cancellation.
//
// GB300 layout: the loop over vectors is sequential, but within a mode step
// the work over the earlier vectors k is independent.  One thread-block
// cluster of up to 16 CTAs runs the whole orthogonalisation in one launch;
// CTA `rank` owns the earlier vectors k = rank (mod cluster) and computes
// their overlaps, products, coefficients and right-hand-side contributions
// (FP64 throughput grows with the number of SMs).  The partial right-hand
// sides meet through distributed shared memory, and every CTA runs the same
// small R x R solve on the same data, so each holds the identical new factor
// and nothing is broadcast back.  One cluster barrier per mode step.
#include <cooperative_groups.h>

#include "common.cuh"
#include "intertwine.cuh"

namespace cg = cooperative_groups;

namespace mlcp {

namespace {

constexpr int kGsThreads = 512;

struct GsSmem {
  double *X, *BB, *Gp, *selfv, *fcs, *bpart, *red, *dinv, *ucol, *misc;
  int* flags;
};

__host__ __device__ inline size_t gs_carve(int R, int npm, GsSmem* s, unsigned char* base) {
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t r = o;
    o += (bytes + 15) / 16 * 16;
    return base ? base + r : nullptr;
  };
  s->X = (double*)take(sizeof(double) * R * npm);
  s->BB = (double*)take(sizeof(double) * R * R);
  s->Gp = (double*)take(sizeof(double) * R * R);
  s->selfv = (double*)take(sizeof(double) * R * npm);
  s->fcs = (double*)take(sizeof(double) * R);
  s->bpart = (double*)take(sizeof(double) * 2 * R * npm);
  s->red = (double*)take(sizeof(double) * kGsThreads / 32);
  s->dinv = (double*)take(sizeof(double) * R);
  s->ucol = (double*)take(sizeof(double) * R);
  s->misc = (double*)take(sizeof(double) * 4);
  s->flags = (int*)take(sizeof(int) * 4);
  return o;
}

__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// Sum over the block (every thread gets the result; red holds one slot per warp).
__device__ double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < nw; ++w) s += red[w];  // same order in every thread
  return s;
}

}  // namespace

__global__ void __launch_bounds__(kGsThreads, 1) gs_kernel(GsParams p) {
  cg::cluster_group cluster = cg::this_cluster();
  const int CL = (int)cluster.num_blocks(), rank = (int)cluster.block_rank();
  const int R = p.R, D = p.D, nD = p.nD, npm = p.npmax, B = p.nbloc, RR = R * R;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid / 32, lane = tid % 32, nwarps = nt / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  GsSmem s;
  gs_carve(R, npm, &s, smem_raw);
  // this CTA's working copy of the vector being orthogonalised and its Grams
  double* fbw = p.work + (size_t)rank * ((size_t)R * nD + (size_t)D * RR);
  double* g64w = fbw + (size_t)R * nD;
  double* psn_all = p.pscr + (size_t)B * D * RR;  // [B][R][R] products over d != j
  auto P = [&](int k, int d) { return p.pscr + ((size_t)k * D + d) * RR; };

  if (tid == 0) s.flags[1] = 0;

  auto load_vector = [&](int iv) {
    const double* fb = p.base + (size_t)iv * R * nD;
    for (int e = tid; e < R * nD; e += nt) fbw[e] = fb[e];
    for (int i = tid; i < R; i += nt) s.fcs[i] = p.coef[(size_t)iv * R + i];
    __syncthreads();
  };
  // FP64 Grams of the working vector, every mode
  auto grams = [&]() {
    for (int e = tid; e < D * RR; e += nt) {
      const int d = e / RR, ii = e % RR, i = ii % R, i2 = ii / R;
      double acc = 0.0;
      for (int q = 0; q < p.nbas[d]; ++q) acc += fbw[(size_t)i * nD + p.off[d] + q] * fbw[(size_t)i2 * nD + p.off[d] + q];
      g64w[e] = acc;
    }
    __syncthreads();
  };
  // weights divided by sqrt(<F,F>)
  auto normalize_weights = [&]() {
    double part = 0.0;
    for (int e = tid; e < RR; e += nt) {
      double prod = s.fcs[e % R] * s.fcs[e / R];
      for (int d = 0; d < D; ++d) prod *= g64w[(size_t)d * RR + e];
      part += prod;
    }
    const double q = sqrt(fabs(block_sum(part, s.red)));
    __syncthreads();
    for (int i = tid; i < R; i += nt) s.fcs[i] /= q;
    __syncthreads();
  };
  auto store_vector = [&](int iv, bool factors) {
    if (rank != 0) return;
    double* fb = p.base + (size_t)iv * R * nD;
    if (factors)
      for (int e = tid; e < R * nD; e += nt) fb[e] = fbw[e];
    for (int i = tid; i < R; i += nt) p.coef[(size_t)iv * R + i] = s.fcs[i];
  };

  load_vector(0);
  grams();
  normalize_weights();
  store_vector(0, false);
  // vector 0's weights are visible to every CTA before they read it as Q_0
  __threadfence();
  cl_arrive();
  cl_wait();

  int step = 0;
  for (int iv = 1; iv < B && p.nals > 0; ++iv) {
    load_vector(iv);
    if (tid == 0) {
      double pen = s.fcs[0];
      for (int i = 1; i < R; ++i) pen = s.fcs[i] > pen ? s.fcs[i] : pen;
      s.misc[0] = pen * 1.0e-10;  // FP64-build rule: this stage is FP64 throughout
    }
    grams();
    // overlaps with the earlier vectors this CTA owns, every mode
    const int nk = (iv - rank + CL - 1) / CL;  // k = rank, rank + CL, ... < iv
    for (size_t e = tid; e < (size_t)nk * D * RR; e += nt) {
      const int kl = (int)(e / ((size_t)D * RR)), rem = (int)(e % ((size_t)D * RR));
      const int k = rank + kl * CL, d = rem / RR, r = (rem % RR) / R, i = rem % R;
      const double* a = p.base + ((size_t)k * R + r) * nD + p.off[d];
      const double* b = fbw + (size_t)i * nD + p.off[d];
      double acc = 0.0;
      for (int q = 0; q < p.nbas[d]; ++q) acc = fma(a[q], b[q], acc);
      P(k, d)[r * R + i] = acc;
    }
    __syncthreads();
    const double pen = s.misc[0];

    for (int it = 0; it < p.nals; ++it) {
      for (int j = 0; j < D; ++j, ++step) {
        const int nj = p.nbas[j];
        double* bp = s.bpart + (size_t)(step & 1) * R * npm;
        // products over d != j for the owned k
        for (size_t e = tid; e < (size_t)nk * RR; e += nt) {
          const int k = rank + (int)(e / RR) * CL, ee = (int)(e % RR);
          double prod = 1.0;
          for (int d = 0; d < D; ++d)
            if (d != j) prod *= P(k, d)[ee];
          psn_all[(size_t)k * RR + ee] = prod;
        }
        // this vector's Grams over d != j: the normal equations and the self term
        for (int e = tid; e < RR; e += nt) {
          double g = 1.0;
          for (int d = 0; d < D; ++d)
            if (d != j) g *= g64w[(size_t)d * RR + e];
          s.Gp[e] = g;
          s.BB[e] = (e % R == e / R) ? g + pen : g;
        }
        __syncthreads();
        // coefficients -<Q_k, F> (one warp per owned k)
        for (int kl = warp; kl < nk; kl += nwarps) {
          const int k = rank + kl * CL;
          const double* qc = p.coef + (size_t)k * R;
          const double* ps = psn_all + (size_t)k * RR;
          const double* pj = P(k, j);
          double part = 0.0;
          for (int ee = lane; ee < RR; ee += 32) part -= qc[ee / R] * s.fcs[ee % R] * ps[ee] * pj[ee];
          for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
          if (lane == 0) p.gcoef[k] = part;
        }
        // self term: sum_r c_r F_r^j(m) prod_{d != j} G_d(r, i)
        for (int e = tid; e < R * nj; e += nt) {
          const int i = e % R, m = e / R;
          double acc = 0.0;
          for (int r = 0; r < R; ++r) acc = fma(s.fcs[r] * fbw[(size_t)r * nD + p.off[j] + m], s.Gp[r * R + i], acc);
          s.selfv[i + m * R] = acc;
        }
        __syncthreads();
        // this CTA's part of sum_k gcoef_k sum_r c_kr Q_kr^j(m) psn_k(r, i)
        for (int e = tid; e < R * nj; e += nt) {
          const int i = e % R, m = e / R;
          double acc = 0.0;
          for (int kl = 0; kl < nk; ++kl) {
            const int k = rank + kl * CL;
            const double* qc = p.coef + (size_t)k * R;
            const double* ps = psn_all + (size_t)k * RR;
            double inner = 0.0;
            for (int r = 0; r < R; ++r)
              inner = fma(qc[r] * p.base[((size_t)k * R + r) * nD + p.off[j] + m], ps[r * R + i], inner);
            acc = fma(p.gcoef[k], inner, acc);
          }
          bp[i + m * R] = acc;
        }
        cl_arrive();
        cl_wait();
        // every CTA: gather in rank order, then the same solve
        for (int e = tid; e < R * nj; e += nt) {
          const int i = e % R, m = e / R;
          double acc = 0.0;
          for (int c = 0; c < CL; ++c) acc += cluster.map_shared_rank(bp, c)[i + m * R];
          s.X[i + m * R] = acc + s.selfv[i + m * R];
        }
        __syncthreads();
        block_ldlt(s.BB, R, R, s.dinv, s.ucol, &s.flags[0]);
        if (tid == 0 && s.flags[0]) s.flags[1] = 1;
        block_ldlt_solve(s.BB, R, R, s.dinv, s.X, nj, R);
        for (int i = tid; i < R; i += nt) {
          double nrm, inv;
          scaled_norm(s.X + i, nj, R, &nrm, &inv);
          for (int m = 0; m < nj; ++m) s.X[i + m * R] *= inv;
          s.fcs[i] = nrm;
        }
        __syncthreads();
        // new factor of mode j, its Gram, and the owned overlaps of mode j
        for (int e = tid; e < R * nj; e += nt) {
          const int i = e / nj, m = e % nj;
          fbw[(size_t)i * nD + p.off[j] + m] = s.X[i + m * R];
        }
        for (int e = tid; e < RR; e += nt) {
          const int i = e % R, i2 = e / R;
          double acc = 0.0;
          for (int q = 0; q < nj; ++q) acc += s.X[i + q * R] * s.X[i2 + q * R];
          g64w[(size_t)j * RR + e] = acc;
        }
        for (size_t e = tid; e < (size_t)nk * RR; e += nt) {
          const int k = rank + (int)(e / RR) * CL, r = (int)(e % RR) / R, i = (int)(e % R);
          const double* a = p.base + ((size_t)k * R + r) * nD + p.off[j];
          double acc = 0.0;
          for (int q = 0; q < nj; ++q) acc = fma(a[q], s.X[i + q * R], acc);
          P(k, j)[r * R + i] = acc;
        }
        __syncthreads();
        normalize_weights();
      }
    }
    // the finished vector becomes Q_iv for the next ones
    store_vector(iv, true);
    __threadfence();
    cl_arrive();
    cl_wait();
  }
  if (rank == 0 && tid == 0 && s.flags[1]) atomicOr(p.status, 1);
  // no CTA leaves while a peer may still read its shared memory
  cl_arrive();
  cl_wait();
}

int gs_cluster_size(int nbloc) { return nbloc > 16 ? 16 : (nbloc > 1 ? nbloc - 1 : 1); }

size_t gs_work_doubles(int nbloc, int R, int nD, int D) {
  return (size_t)gs_cluster_size(nbloc) * ((size_t)R * nD + (size_t)D * R * R);
}

int gs_launch(const GsParams& p, cudaStream_t st) {
  GsSmem s;
  const size_t smem = gs_carve(p.R, p.npmax, &s, nullptr);
  const int cl = gs_cluster_size(p.nbloc);
  MLCP_CUDA_TRY(cudaFuncSetAttribute(gs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (cl > 8) MLCP_CUDA_TRY(cudaFuncSetAttribute(gs_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(cl);
  cfg.blockDim = dim3(kGsThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cl;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MLCP_CUDA_TRY(cudaLaunchKernelEx(&cfg, gs_kernel, p));
  return kOk;
}

}  // namespace mlcp
