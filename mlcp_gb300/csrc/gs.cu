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
// The loop over vectors is inherently sequential; the whole orthogonalisation
// is one launch.
#include "common.cuh"
#include "intertwine.cuh"

namespace mlcp {

namespace {
constexpr int kGsThreads = 512;
}

__global__ void __launch_bounds__(kGsThreads) gs_kernel(GsParams p) {
  const int R = p.R, D = p.D, nD = p.nD, nDp = p.nDp, npm = p.npmax, B = p.nbloc;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int warp = tid / 32, lane = tid % 32, nwarps = nt / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* ptr = smem_raw;
  auto take = [&](size_t bytes) { unsigned char* r = ptr; ptr += (bytes + 15) / 16 * 16; return r; };
  double* X = (double*)take(sizeof(double) * R * npm);
  double* BB = (double*)take(sizeof(double) * R * R);
  double* cf = (double*)take(sizeof(double) * R);
  double* red = (double*)take(sizeof(double) * nt);
  double* dinv = (double*)take(sizeof(double) * R);
  double* ucol = (double*)take(sizeof(double) * R);
  int* flags = (int*)take(sizeof(int) * 4);

  double* psn = p.pscr + (size_t)B * D * R * R;  // [B][R][R] products over d != j

  for (int k = tid; k < B; k += nt) p.gcoef[k] = 1.0;
  if (tid == 0) flags[1] = 0;
  __syncthreads();

  // <F,F> from FP64 Grams of vector iv -> weights / sqrt(norm)
  auto grams_of = [&](int iv) {
    const double* fb = p.base + (size_t)iv * R * nD;
    for (int e = tid; e < D * R * R; e += nt) {
      const int d = e / (R * R), ii = e % (R * R), i = ii % R, i2 = ii / R;
      double acc = 0.0;
      for (int q = 0; q < p.nbas[d]; ++q) acc += fb[(size_t)i * nD + p.off[d] + q] * fb[(size_t)i2 * nD + p.off[d] + q];
      p.g64[e] = acc;
    }
  };
  auto normalize_weights = [&](int iv) {
    double* fc = p.coef + (size_t)iv * R;
    double part = 0.0;
    for (int e = tid; e < R * R; e += nt) {
      double prod = fc[e % R] * fc[e / R];
      for (int d = 0; d < D; ++d) prod *= p.g64[(size_t)d * R * R + e];
      part += prod;
    }
    red[tid] = part;
    __syncthreads();
    if (tid == 0) {
      double s = 0.0;
      for (int k = 0; k < nt; ++k) s += red[k];
      red[0] = sqrt(fabs(s));
    }
    __syncthreads();
    const double q = red[0];
    __syncthreads();
    for (int i = tid; i < R; i += nt) fc[i] /= q;
    __syncthreads();
  };

  grams_of(0);
  __syncthreads();
  normalize_weights(0);

  for (int iv = 1; iv < B && p.nals > 0; ++iv) {
    double* fb = p.base + (size_t)iv * R * nD;
    double* fc = p.coef + (size_t)iv * R;
    if (tid == 0) {
      double pen = fc[0];
      for (int i = 1; i < R; ++i) pen = fc[i] > pen ? fc[i] : pen;
      red[0] = pen * 1.0e-10;  // FP64-build rule: this stage is FP64 throughout
    }
    grams_of(iv);
    // overlaps with every earlier vector, every mode
    for (size_t e = tid; e < (size_t)iv * D * R * R; e += nt) {
      const int k = (int)(e / ((size_t)D * R * R));
      const int rem = (int)(e % ((size_t)D * R * R));
      const int d = rem / (R * R), r = (rem % (R * R)) / R, i = rem % R;
      const double* a = p.base + ((size_t)k * R + r) * nD + p.off[d];
      const double* b = fb + (size_t)i * nD + p.off[d];
      double acc = 0.0;
      for (int q = 0; q < p.nbas[d]; ++q) acc = fma(a[q], b[q], acc);
      p.pscr[((size_t)k * D + d) * R * R + r * R + i] = acc;
    }
    __syncthreads();
    const double pen = red[0];
    __syncthreads();

    for (int it = 0; it < p.nals; ++it) {
      for (int j = 0; j < D; ++j) {
        const int nj = p.nbas[j];
        // products over d != j and the coefficients -<Q_k, F> (one warp per k)
        for (size_t e = tid; e < (size_t)iv * R * R; e += nt) {
          const int k = (int)(e / (R * R)), ee = (int)(e % (R * R));
          double prod = 1.0;
          for (int d = 0; d < D; ++d)
            if (d != j) prod *= p.pscr[((size_t)k * D + d) * R * R + ee];
          psn[(size_t)k * R * R + ee] = prod;
        }
        __syncthreads();
        for (int k = warp; k < iv; k += nwarps) {
          const double* qc = p.coef + (size_t)k * R;
          double part = 0.0;
          for (int ee = lane; ee < R * R; ee += 32) {
            const int r = ee / R, i = ee % R;
            part -= qc[r] * fc[i] * psn[(size_t)k * R * R + ee] * p.pscr[((size_t)k * D + j) * R * R + ee];
          }
          for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
          if (lane == 0) p.gcoef[k] = part;
        }
        __syncthreads();
        // right-hand side: sum_k gcoef[k] sum_r c_r Q_{k,r}^j(n) psn_k(r,i) + F self term
        for (int e = tid; e < R * nj; e += nt) {
          const int i = e % R, m = e / R;
          double acc = 0.0;
          for (int k = 0; k < iv; ++k) {
            const double* qc = p.coef + (size_t)k * R;
            double inner = 0.0;
            for (int r = 0; r < R; ++r)
              inner = fma(qc[r] * p.base[((size_t)k * R + r) * nD + p.off[j] + m], psn[(size_t)k * R * R + r * R + i],
                          inner);
            acc += p.gcoef[k] * inner;
          }
          double self = 0.0;
          for (int r = 0; r < R; ++r) {
            double prod = fc[r] * fb[(size_t)r * nD + p.off[j] + m];
            for (int d = 0; d < D; ++d)
              if (d != j) prod *= p.g64[(size_t)d * R * R + r * R + i];
            self += prod;
          }
          X[i + m * R] = acc + p.gcoef[iv] * self;
        }
        for (int e = tid; e < R * R; e += nt) {
          double bb = 1.0;
          for (int d = 0; d < D; ++d)
            if (d != j) bb *= p.g64[(size_t)d * R * R + e];
          if (e % R == e / R) bb += pen;
          BB[e] = bb;
        }
        __syncthreads();
        block_ldlt(BB, R, R, dinv, ucol, &flags[0]);
        if (tid == 0 && flags[0]) flags[1] = 1;
        block_ldlt_solve(BB, R, R, dinv, X, nj, R);
        for (int i = tid; i < R; i += nt) {
          double nrm, inv;
          scaled_norm(X + i, nj, R, &nrm, &inv);
          for (int m = 0; m < nj; ++m) X[i + m * R] *= inv;
          fc[i] = nrm;
        }
        __syncthreads();
        for (int e = tid; e < R * nj; e += nt) {
          const int i = e / nj, m = e % nj;
          fb[(size_t)i * nD + p.off[j] + m] = X[i + m * R];
        }
        __syncthreads();
        // refresh Gram and overlaps of mode j
        for (int e = tid; e < R * R; e += nt) {
          const int i = e % R, i2 = e / R;
          double acc = 0.0;
          for (int q = 0; q < nj; ++q) acc += fb[(size_t)i * nD + p.off[j] + q] * fb[(size_t)i2 * nD + p.off[j] + q];
          p.g64[(size_t)j * R * R + e] = acc;
        }
        for (size_t e = tid; e < (size_t)iv * R * R; e += nt) {
          const int k = (int)(e / (R * R)), r = (int)(e % (R * R)) / R, i = (int)(e % R);
          const double* a = p.base + ((size_t)k * R + r) * nD + p.off[j];
          const double* b = fb + (size_t)i * nD + p.off[j];
          double acc = 0.0;
          for (int q = 0; q < nj; ++q) acc = fma(a[q], b[q], acc);
          p.pscr[((size_t)k * D + j) * R * R + r * R + i] = acc;
        }
        __syncthreads();
        normalize_weights(iv);
      }
    }
  }
  if (tid == 0 && flags[1]) atomicOr(p.status, 1);
}

int gs_launch(const GsParams& p, cudaStream_t st) {
  size_t smem = 0;
  auto take = [&](size_t bytes) { smem += (bytes + 15) / 16 * 16; };
  take(sizeof(double) * p.R * p.npmax);
  take(sizeof(double) * p.R * p.R);
  take(sizeof(double) * p.R);
  take(sizeof(double) * kGsThreads);
  take(sizeof(double) * p.R);
  take(sizeof(double) * p.R);
  take(sizeof(int) * 4);
  MLCP_CUDA_TRY(cudaFuncSetAttribute(gs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  gs_kernel<<<1, kGsThreads, smem, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp
