// ALS-fitted Hamiltonian applications, one persistent CTA per vector.
//
// Reference: POW_ALS (src/intertw_mvp.cu:452-497) and PRODHV_ALS (:501-549)
// with mvp_build_linear_system (:380-448).  For mode j the reference builds,
// for every term t, G = h_t Fo (all modes, mvp_kernel :39), then
// PS = prod_{d!=j} <G^d, F^d> (constpstot) and accumulates
// b(i,n) += sum_r c_r G_r^j(n) PS(r,i) (constbjk): 3T launches per mode step.
//
// Here the same b is assembled from per-mode operator Grams
//   M[d][u](r,i) = <h_u Fo_r^d, F_i^d>     (one R x R matrix per distinct operator u of mode d)
// which change only when mode d of F changes:
//   W_u = sum_{t: op(t,j) = u} alpha_t prod_{d!=j} M[d][op(t,d)]
//   b(i,n) = sum_u sum_r c_r W_u(r,i) (h_u Fo_r^j)(n)
// so a mode step costs O(T R^2 D) instead of O(T R (sum_d n_d^2 + R nD)).
// The energy shift enters as an identity term with weight -E; for ishift < 0
// b changes sign, as in the reference.  Because the right-hand sides carry
// FP32 rounding, the penalty follows the reference's FP32-build rule
// (1e-5 max c, src/als.cu:248-267): with the FP64 rule (1e-10) the rounding
// noise in near-null directions of the normal equations is amplified by up
// to 1e10 and the CP weights blow up over successive cycles.  The R x R normal equations
// (prod_{d!=j} F_d F_d^T + pen I), their Cholesky solve, the F Grams and the
// weight normalisation run in FP64; the operator Grams, term products and
// right-hand sides run in FP32.
#include "common.cuh"
#include "intertwine.cuh"

namespace mlcp {

namespace {

constexpr int kThreads = 256;

struct OpSmem {
  float* f32;     // [R][nDp] current F (FP32)
  float* fo32;    // [R][nDp] Fo (FP32); aliases f32 for POW
  float* y;       // [R][npmax] temporary h Fo_r
  double* X;      // [R][npmax] right-hand side / solution (column-major, ld R)
  double* BB;     // [R][R]
  double* cf;     // [R] weights of F
  double* cfo;    // [R] weights of Fo
  double* red;    // [kThreads] reduction scratch
  double* dinv;   // [R] reciprocal pivots
  double* u;      // [R] LDL^T scratch column
  int* flags;     // [4]
};

__device__ inline void carve(OpSmem& s, unsigned char* base, const OpTable& t, bool separate_fo) {
  unsigned char* ptr = base;
  auto take = [&](size_t bytes) { unsigned char* r = ptr; ptr += (bytes + 15) / 16 * 16; return r; };
  s.f32 = (float*)take(sizeof(float) * t.R * t.nDp);
  s.fo32 = separate_fo ? (float*)take(sizeof(float) * t.R * t.nDp) : s.f32;
  s.y = (float*)take(sizeof(float) * t.R * t.npmax);
  s.X = (double*)take(sizeof(double) * t.R * t.npmax);
  s.BB = (double*)take(sizeof(double) * t.R * t.R);
  s.cf = (double*)take(sizeof(double) * t.R);
  s.cfo = (double*)take(sizeof(double) * t.R);
  s.red = (double*)take(sizeof(double) * kThreads);
  s.dinv = (double*)take(sizeof(double) * t.R);
  s.u = (double*)take(sizeof(double) * t.R);
  s.flags = (int*)take(sizeof(int) * 4);
}

// M(r,i) = sum_n (h Fo_r^d)(n) F_i^d(n); identity operators skip the product.
__device__ void operator_gram(const OpTable& t, int d, int ug, const OpSmem& s, float* M, float* zout) {
  const int R = t.R, n = t.nbas[d], op = t.offp[d], npm = t.npmax;
  const bool ident = t.ident[ug];
  const float* h = t.hmat + (size_t)ug * npm * npm;
  // y(r, m) = sum_k h(m, k) Fo_r(k)
  for (int e = threadIdx.x; e < R * n; e += blockDim.x) {
    const int r = e / n, m = e % n;
    float acc;
    if (ident) {
      acc = s.fo32[r * t.nDp + op + m];
    } else {
      acc = 0.f;
      for (int k = 0; k < n; ++k) acc = fmaf(h[m * npm + k], s.fo32[r * t.nDp + op + k], acc);
    }
    s.y[r * npm + m] = acc;
    if (zout) zout[r * npm + m] = acc;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
    const int r = e / R, i = e % R;
    float acc = 0.f;
    for (int m = 0; m < n; ++m) acc = fmaf(s.y[r * npm + m], s.f32[i * t.nDp + op + m], acc);
    M[e] = acc;
  }
  __syncthreads();
}

// FP64 Gram of mode d of F (global FP64 factors).
__device__ void f_gram64(const OpTable& t, int d, const double* fb, int nD, double* G) {
  const int R = t.R, n = t.nbas[d], o = t.off[d];
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
    const int i = e % R, i2 = e / R;
    double acc = 0.0;
    for (int q = 0; q < n; ++q) acc += fb[(size_t)i * nD + o + q] * fb[(size_t)i2 * nD + o + q];
    G[e] = acc;
  }
}

}  // namespace

__global__ void __launch_bounds__(kThreads) opals_kernel(OpAlsParams p) {
  const OpTable& t = p.ops;
  const int v = blockIdx.x;
  const int R = t.R, D = t.D, T = t.T, npm = t.npmax, nD = p.nD;
  const bool pow_mode = (p.mode == 0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  OpSmem s;
  carve(s, smem_raw, t, !pow_mode);

  const double* fob = p.fo_base + (size_t)v * R * nD;
  const double* foc = p.fo_coef + (size_t)v * R;
  double* fb = p.f_base + (size_t)v * R * nD;
  double* fc = p.f_coef + (size_t)v * R;
  float* M = p.mscr + (size_t)v * t.utot * R * R;
  float* W = p.wscr + (size_t)v * t.umax * R * R;
  float* Z = p.zscr + (size_t)v * t.umax * R * npm;
  double* G64 = p.g64 + (size_t)v * D * R * R;

  // ---- set-up: F (= Fo for PRODHV), FP32 copies, Grams, penalty ----
  if (!pow_mode) {
    for (int e = threadIdx.x; e < R * nD; e += blockDim.x) fb[e] = fob[e];
    for (int e = threadIdx.x; e < R; e += blockDim.x) fc[e] = foc[e];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < R * t.nDp; e += blockDim.x) {
    const int r = e / t.nDp, q = e % t.nDp;
    int d = 0;
    while (d + 1 < D && t.offp[d + 1] <= q) ++d;
    const int k = q - t.offp[d];
    const double x = (k < t.nbas[d]) ? fob[(size_t)r * nD + t.off[d] + k] : 0.0;
    s.f32[e] = (float)x;
    if (!pow_mode) s.fo32[e] = (float)x;
  }
  for (int e = threadIdx.x; e < R; e += blockDim.x) {
    s.cf[e] = fc[e];
    s.cfo[e] = foc[e];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double pen = s.cfo[0];
    for (int i = 1; i < R; ++i) pen = s.cfo[i] > pen ? s.cfo[i] : pen;
    s.red[0] = pen * p.pen_factor;
    s.flags[0] = 0;
    s.flags[1] = 0;
  }
  for (int d = 0; d < D; ++d) f_gram64(t, d, fb, nD, G64 + (size_t)d * R * R);
  __syncthreads();
  const double pen = s.red[0];
  for (int d = 0; d < D; ++d)
    for (int u = 0; u < t.uoff[d + 1] - t.uoff[d]; ++u)
      operator_gram(t, d, t.uoff[d] + u, s, M + (size_t)(t.uoff[d] + u) * R * R, nullptr);

  for (int sw = 0; sw < p.nsweeps; ++sw) {
    for (int j = 0; j < D; ++j) {
      const int nj = t.nbas[j], opj = t.offp[j];
      const int nu = t.uoff[j + 1] - t.uoff[j];
      const int* ord = t.order + (size_t)j * T;
      const int* gs = t.gstart + (size_t)j * (t.umax + 1);
      // -- grouped term products W_u --
      for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        for (int u = 0; u < nu; ++u) {
          float acc = 0.f;
          for (int q = gs[u]; q < gs[u + 1]; ++q) {
            const int term = ord[q];
            float prod = (float)t.alpha[term];
            const int* ut = t.uid + (size_t)term * D;
            for (int d = 0; d < D; ++d) {
              if (d == j) continue;
              prod *= M[(size_t)(t.uoff[d] + ut[d]) * R * R + e];
            }
            acc += prod;
          }
          if (u == 0 && p.ishift != 0) {
            float prod = (float)(-(p.eshift_v ? p.eshift_v[v] : p.eshift));
            for (int d = 0; d < D; ++d)
              if (d != j) prod *= M[(size_t)t.uoff[d] * R * R + e];
            acc += prod;
          }
          W[(size_t)u * R * R + e] = acc;
        }
      }
      // -- h_u Fo_j for every operator of mode j --
      for (int u = 0; u < nu; ++u) {
        const int ug = t.uoff[j] + u;
        const float* h = t.hmat + (size_t)ug * npm * npm;
        for (int e = threadIdx.x; e < R * nj; e += blockDim.x) {
          const int r = e / nj, m = e % nj;
          float acc;
          if (t.ident[ug]) {
            acc = s.fo32[r * t.nDp + opj + m];
          } else {
            acc = 0.f;
            for (int k = 0; k < nj; ++k) acc = fmaf(h[m * npm + k], s.fo32[r * t.nDp + opj + k], acc);
          }
          Z[(size_t)u * R * npm + r * npm + m] = acc;
        }
      }
      __syncthreads();
      // -- right-hand side b(i,n) = sum_u sum_r W_u(r,i) c_r Z_u(r,n) --
      const double* cg = pow_mode ? s.cf : s.cfo;
      for (int e = threadIdx.x; e < R * nj; e += blockDim.x) {
        const int i = e % R, m = e / R;
        float acc = 0.f;
        for (int u = 0; u < nu; ++u)
          for (int r = 0; r < R; ++r)
            acc = fmaf(W[(size_t)u * R * R + r * R + i] * (float)cg[r], Z[(size_t)u * R * npm + r * npm + m], acc);
        double b = (double)acc;
        if (p.ishift < 0) b = -b;
        s.X[i + m * R] = b;
      }
      // -- FP64 normal equations --
      for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        double bb = 1.0;
        for (int d = 0; d < D; ++d)
          if (d != j) bb *= G64[(size_t)d * R * R + e];
        if (e % R == e / R) bb += pen;
        s.BB[e] = bb;
      }
      __syncthreads();
      block_ldlt(s.BB, R, R, s.dinv, s.u, &s.flags[2]);
      if (threadIdx.x == 0 && s.flags[2]) s.flags[1] = 1;
      block_ldlt_solve(s.BB, R, R, s.dinv, s.X, nj, R);
      for (int i = threadIdx.x; i < R; i += blockDim.x) {
        double nrm, inv;
        scaled_norm(s.X + i, nj, R, &nrm, &inv);
        for (int m = 0; m < nj; ++m) s.X[i + m * R] *= inv;
        s.cf[i] = nrm;
        fc[i] = nrm;
      }
      __syncthreads();
      for (int e = threadIdx.x; e < R * nj; e += blockDim.x) {
        const int i = e / nj, m = e % nj;
        const double x = s.X[i + m * R];
        fb[(size_t)i * nD + t.off[j] + m] = x;
        s.f32[i * t.nDp + opj + m] = (float)x;
      }
      __syncthreads();
      f_gram64(t, j, fb, nD, G64 + (size_t)j * R * R);
      // -- operator Grams of mode j with the new factor --
      for (int u = 0; u < nu; ++u) {
        const int ug = t.uoff[j] + u;
        float* Mu = M + (size_t)ug * R * R;
        if (pow_mode) {
          operator_gram(t, j, ug, s, Mu, nullptr);
        } else {
          // Fo is fixed: h_u Fo_j is still in Z
          for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
            const int r = e / R, i = e % R;
            float acc = 0.f;
            for (int m = 0; m < nj; ++m)
              acc = fmaf(Z[(size_t)u * R * npm + r * npm + m], s.f32[i * t.nDp + opj + m], acc);
            Mu[e] = acc;
          }
        }
      }
      __syncthreads();
    }
    if (pow_mode) {
      // weight renormalisation after each sweep (src/intertw_mvp.cu:491-494)
      double part = 0.0;
      for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        double prod = s.cf[e % R] * s.cf[e / R];
        for (int d = 0; d < D; ++d) prod *= G64[(size_t)d * R * R + e];
        part += prod;
      }
      s.red[threadIdx.x] = part;
      __syncthreads();
      if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int k = 0; k < blockDim.x; ++k) tot += s.red[k];
        s.red[0] = sqrt(fabs(tot));
      }
      __syncthreads();
      const double q = s.red[0];
      __syncthreads();
      for (int i = threadIdx.x; i < R; i += blockDim.x) {
        s.cf[i] /= q;
        fc[i] = s.cf[i];
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0 && s.flags[1]) atomicOr(&p.status[v], 1);
}

size_t opals_smem_bytes(const OpTable& t) {
  size_t b = 0;
  auto take = [&](size_t bytes) { b += (bytes + 15) / 16 * 16; };
  take(sizeof(float) * t.R * t.nDp);
  take(sizeof(float) * t.R * t.nDp);
  take(sizeof(float) * t.R * t.npmax);
  take(sizeof(double) * t.R * t.npmax);
  take(sizeof(double) * t.R * t.R);
  take(sizeof(double) * t.R);
  take(sizeof(double) * t.R);
  take(sizeof(double) * kThreads);
  take(sizeof(double) * t.R);
  take(sizeof(double) * t.R);
  take(sizeof(int) * 4);
  return b;
}

int opals_launch(const OpAlsParams& p, cudaStream_t st) {
  const size_t smem = opals_smem_bytes(p.ops);
  MLCP_CUDA_TRY(cudaFuncSetAttribute(opals_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  opals_kernel<<<p.nvec, kThreads, smem, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp
