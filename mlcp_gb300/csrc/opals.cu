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
// b changes sign, as in the reference.
//
// Precision.  The penalty is the reference's FP64-build rule (1e-10 max c,
// src/als.cu:248-267).  With it the normal equations of a nearly converged
// vector (whose terms are close to linearly dependent) have condition
// numbers up to 1e10, so any noise in b along their near-null directions is
// amplified by up to 1e10: FP32 right-hand sides (24 bits) made the weights
// blow up over successive cycles.  Everything here therefore runs in
// double-word arithmetic (dword.cuh, about 48 bits): the factors of F and Fo,
// the operators, the operator Grams M, the term products W, h_u Fo_j, the
// right-hand sides, the normal equations (prod_{d!=j} F_d F_d^T + pen I),
// their solve (FP32 inverse as the preconditioner of a double-word
// refinement, or a double-word LDL^T), the F Grams and the weight
// normalisation; the factors are written out in FP64.  In POW the weights
// are rescaled by a power of two after every mode step
// (rescale_weights_warp), which keeps them in the FP32 exponent range of
// the double-word values without changing the sweep's result.
#include "common.cuh"
#include "dword.cuh"
#include "dwsolve.cuh"
#include "intertwine.cuh"

namespace mlcp {

namespace {

constexpr int kThreads = 256;

constexpr int kWarps = kThreads / 32;

struct OpSmem {
  dw* f;          // [R][nDp] current F
  dw* fo;         // [R][nDp] Fo; aliases f for POW
  dw* y;          // [R][npmax] temporary h Fo_r
  dw* X;          // [R][npmax] solution (column-major, ld R)
  dw* b0;         // [R][npmax] right-hand side
  dw* res;        // [R][npmax] refinement residual
  dw* BB;         // [R][R] normal equations
  float* gi;      // [2][R][R] FP32 inverse of BB
  dw* cf;         // [R] weights of F
  dw* cfo;        // [R] weights of Fo
  dw* red;        // [kWarps] reduction scratch
  dw* dinv;       // [R] LDL^T reciprocal pivots
  dw* u;          // [R] LDL^T scratch column
  dw* misc;       // [2] penalty, norm
  float* rred;    // [4] refinement scratch
  dwsolve::ColScratch cs;
  int* moff;      // [T][D] offset of each term's operator Gram per mode (null when T D is large)
  int* ord;       // [D][T] terms grouped by their operator at each mode (with moff)
  int* gst;       // [D][umax+1] group starts (with moff)
  dw* alpha;      // [T] term coefficients (with moff)
  dw *Ms, *Ws, *Zs;  // operator Grams, term products, h_u Fo_j when resident in shared memory
  dw* hs;         // [utot][npmax][npmax] the operators when resident
  int* flags;     // [4]
};

// Terms x modes up to which the Gram offsets are tabulated in shared memory.
constexpr int kMoffMax = 8192;

// Carves the shared memory (null base: sizes only); returns the bytes.
// tabulate: copy the term tables (Gram offsets, operator groups, term
// coefficients) into shared memory when T D <= kMoffMax; without them the
// kernel reads the same tables from the global operator table.
__host__ __device__ inline size_t carve(OpSmem& s, unsigned char* base, const OpTable& t, bool separate_fo,
                                        bool resident, bool tabulate) {
  size_t o = 0;
  auto take = [&](size_t bytes) -> unsigned char* {
    const size_t r = o;
    o += (bytes + 15) / 16 * 16;
    return base ? base + r : nullptr;
  };
  const size_t Rn = (size_t)t.R * t.npmax, RR = (size_t)t.R * t.R;
  s.f = (dw*)take(sizeof(dw) * t.R * t.nDp);
  s.fo = separate_fo ? (dw*)take(sizeof(dw) * t.R * t.nDp) : s.f;
  s.y = (dw*)take(sizeof(dw) * Rn);
  s.X = (dw*)take(sizeof(dw) * Rn);
  s.b0 = (dw*)take(sizeof(dw) * Rn);
  s.res = (dw*)take(sizeof(dw) * Rn);
  s.BB = (dw*)take(sizeof(dw) * RR);
  s.gi = (float*)take(sizeof(float) * 2 * RR);
  s.cf = (dw*)take(sizeof(dw) * t.R);
  s.cfo = (dw*)take(sizeof(dw) * t.R);
  s.red = (dw*)take(sizeof(dw) * kWarps);
  s.dinv = (dw*)take(sizeof(dw) * t.R);
  s.u = (dw*)take(sizeof(dw) * t.R);
  s.misc = (dw*)take(sizeof(dw) * 2);
  s.rred = (float*)take(sizeof(float) * 4);
  s.cs.conv = (float*)take(sizeof(float) * 64);
  s.cs.rmax = (float*)take(sizeof(float) * 16 * 32);
  s.cs.rsum = (dw*)take(sizeof(dw) * 16 * 32);
  const bool tab = tabulate && t.T * t.D <= kMoffMax;
  s.moff = tab ? (int*)take(sizeof(int) * t.T * t.D) : nullptr;
  s.ord = tab ? (int*)take(sizeof(int) * t.T * t.D) : nullptr;
  s.gst = tab ? (int*)take(sizeof(int) * t.D * (t.umax + 1)) : nullptr;
  s.alpha = tab ? (dw*)take(sizeof(dw) * t.T) : nullptr;
  s.hs = resident ? (dw*)take(sizeof(dw) * t.utot * t.npmax * t.npmax) : nullptr;
  s.Ms = resident ? (dw*)take(sizeof(dw) * t.utot * RR) : nullptr;
  s.Ws = resident ? (dw*)take(sizeof(dw) * t.umax * RR) : nullptr;
  s.Zs = resident ? (dw*)take(sizeof(dw) * t.umax * Rn) : nullptr;
  s.flags = (int*)take(sizeof(int) * 4);
  return o;
}

// Sum over the block; thread 0 gets the result (fixed order).
__device__ dw block_sum_dw(dw v, dw* red) {
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

// In-place POW applies (H - E) once per mode step, so within a sweep the
// weights grow (or shrink) by about ||H - E|| per step: a 12-mode quartic
// force field in cm^-1 passes the FP32 exponent range after nine steps, and a
// 400-term random Hamiltonian over 24 modes overflows the squared row norms
// (weights above 1.8e19).  The end-of-sweep renormalisation divides out any
// common factor, so after each step the weights are multiplied by the power
// of two that brings the largest into [0.5, 1): exact, and the solve is linear
// in the weights, so the sweep's result is unchanged.  Warp 0 only; each lane
// rescales the entries it read.
__device__ void rescale_weights_warp(dw* cf, int R) {
  float m = 0.f;
  for (int i = threadIdx.x; i < R; i += 32) m = fmaxf(m, fabsf(cf[i].hi));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (!(m > 0.f && m <= 3.4028235e38f)) return;  // zero, or non-finite (reported by the next solve)
  int e;
  frexpf(m, &e);
  for (int i = threadIdx.x; i < R; i += 32) cf[i] = dw_make(ldexpf(cf[i].hi, -e), ldexpf(cf[i].lo, -e));
}

// M(r,i) = sum_n (h Fo_r^d)(n) F_i^d(n); identity operators skip the product.
__device__ void operator_gram(const OpTable& t, const dw* hmat, int d, int ug, const OpSmem& s, dw* M) {
  const int R = t.R, n = t.nbas[d], op = t.offp[d], npm = t.npmax;
  const bool ident = t.ident[ug];
  const dw* h = hmat + (size_t)ug * npm * npm;
  // y(r, m) = sum_k h(m, k) Fo_r(k)
  for (int e = threadIdx.x; e < R * n; e += blockDim.x) {
    const int r = e / n, m = e % n;
    dw val;
    if (ident) {
      val = s.fo[r * t.nDp + op + m];
    } else {
      dw_acc acc = acc_zero();
      for (int k = 0; k < n; ++k) acc_fma(acc, h[m * npm + k], s.fo[r * t.nDp + op + k]);
      val = acc_value(acc);
    }
    s.y[r * npm + m] = val;
  }
  __syncthreads();
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
    const int r = e / R, i = e % R;
    dw_acc acc = acc_zero();
    for (int m = 0; m < n; ++m) acc_fma(acc, s.y[r * npm + m], s.f[i * t.nDp + op + m]);
    M[e] = acc_value(acc);
  }
  __syncthreads();
}

// Double-word Gram of mode d of F from the FP64 factors (set-up only).
__device__ void f_gram_from64(const OpTable& t, int d, const double* fb, int nD, dw* G) {
  const int R = t.R, n = t.nbas[d], o = t.off[d];
  for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
    const int i = e % R, i2 = e / R;
    double acc = 0.0;
    for (int q = 0; q < n; ++q) acc += fb[(size_t)i * nD + o + q] * fb[(size_t)i2 * nD + o + q];
    G[e] = dw_from_double(acc);
  }
}

}  // namespace

// kResident: the operator Grams, term products, h_u Fo_j and the operators in
// shared memory (else in the per-vector global scratch of p and the table).
template <bool kResident>
__global__ void __launch_bounds__(kThreads, 1) opals_kernel(OpAlsParams p) {
  const OpTable& t = p.ops;
  const int v = blockIdx.x;
  const int R = t.R, D = t.D, T = t.T, npm = t.npmax, nD = p.nD, RR = R * R;
  const bool pow_mode = (p.mode == 0);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  OpSmem s;
  carve(s, smem_raw, t, !pow_mode, kResident, p.tabulate != 0);

  const double* fob = p.fo_base + (size_t)v * R * nD;
  const double* foc = p.fo_coef + (size_t)v * R;
  double* fb = p.f_base + (size_t)v * R * nD;
  double* fc = p.f_coef + (size_t)v * R;
  dw* M = kResident ? s.Ms : p.mscr + (size_t)v * t.utot * R * R;
  dw* W = kResident ? s.Ws : p.wscr + (size_t)v * t.umax * R * R;
  dw* Z = kResident ? s.Zs : p.zscr + (size_t)v * t.umax * R * npm;
  const int* moff = s.moff;
  if (moff) {
    for (int e = threadIdx.x; e < T * D; e += blockDim.x) {
      s.moff[e] = (t.uoff[e % D] + t.uid[e]) * RR;
      s.ord[e] = t.order[e];
    }
    for (int e = threadIdx.x; e < D * (t.umax + 1); e += blockDim.x) s.gst[e] = t.gstart[e];
    for (int e = threadIdx.x; e < T; e += blockDim.x) s.alpha[e] = dw_from_double(t.alpha[e]);
  }
  const dw* hmat = kResident ? s.hs : t.hdw;
  if (kResident)
    for (int e = threadIdx.x; e < t.utot * npm * npm; e += blockDim.x) s.hs[e] = t.hdw[e];
  dw* G = reinterpret_cast<dw*>(p.g64) + (size_t)v * D * R * R;  // double-word F Grams per mode

  // ---- set-up: F (= Fo for PRODHV), double-word copies, Grams, penalty ----
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
    const dw x = dw_from_double((k < t.nbas[d]) ? fob[(size_t)r * nD + t.off[d] + k] : 0.0);
    s.f[e] = x;
    if (!pow_mode) s.fo[e] = x;
  }
  for (int e = threadIdx.x; e < R; e += blockDim.x) {
    s.cf[e] = dw_from_double(fc[e]);
    s.cfo[e] = dw_from_double(foc[e]);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double pen = foc[0];
    for (int i = 1; i < R; ++i) pen = foc[i] > pen ? foc[i] : pen;
    s.misc[0] = dw_from_double(pen * p.pen_factor);
    s.flags[0] = 0;
    s.flags[1] = 0;
  }
  for (int d = 0; d < D; ++d) f_gram_from64(t, d, fb, nD, G + (size_t)d * R * R);
  __syncthreads();
  const dw pen = s.misc[0];
  const int rv = p.rank_v ? p.rank_v[v] : R;  // ragged: this vector's rank
  for (int d = 0; d < D; ++d)
    for (int u = 0; u < t.uoff[d + 1] - t.uoff[d]; ++u)
      operator_gram(t, hmat, d, t.uoff[d] + u, s, M + (size_t)(t.uoff[d] + u) * R * R);
  const dw eshift = dw_from_double(-(p.eshift_v ? p.eshift_v[v] : p.eshift));

  for (int sw = 0; sw < p.nsweeps; ++sw) {
    for (int j = 0; j < D; ++j) {
      const int nj = t.nbas[j], opj = t.offp[j];
      const int nu = t.uoff[j + 1] - t.uoff[j];
      const int* ord = (moff ? s.ord : t.order) + (size_t)j * T;
      const int* gs = (moff ? s.gst : t.gstart) + (size_t)j * (t.umax + 1);
      // -- normal equations from the Grams of the previous step:
      //    prod_{d != j} G_d + pen I --
      for (int e = threadIdx.x; e < RR; e += blockDim.x) {
        dw bb = dw_make(1.f);
        for (int d = 0; d < D; ++d)
          if (d != j) bb = dw_mul(bb, G[(size_t)d * RR + e]);
        if (e % R == e / R) bb = dw_add(bb, pen);
        if (e % R >= rv || e / R >= rv) bb = dw_make(e % R == e / R ? 1.f : 0.f);  // ragged: decoupled padding
        s.BB[e] = bb;
      }
      __syncthreads();
      // -- their FP32 inverse (warp 0 in registers for R <= 32, else warps
      //    0-3) while the other warps form the right-hand side --
      const int w0 = R <= 32 ? 32 : dwsolve::kSolverThreads;
      if (threadIdx.x < w0) {
        if (R <= 32) {
          const bool g = dwsolve::gj_inverse_warp(s.BB, R, s.gi);
          if (threadIdx.x == 0) {
            s.flags[2] = g;
            s.flags[0] = 0;
          }
        } else {
          bool ok;
          const float* iv = dwsolve::gj_inverse(s.BB, R, s.gi, &ok);
          if (threadIdx.x == 0) {
            s.flags[2] = ok;
            s.flags[0] = iv == s.gi ? 0 : 1;
          }
        }
      } else {
        const int wt = threadIdx.x - w0, nw = kThreads - w0;
        // grouped term products W_u(r,i) = sum_{t in group u} alpha_t prod_{d != j} M[d][op(t,d)](r,i),
        // four terms at a time
        for (int item = wt; item < nu * RR; item += nw) {
          const int u = item / RR, e = item - u * RR;
          dw_acc acc = acc_zero();
          for (int q = gs[u]; q < gs[u + 1]; q += 4) {
            dw pr[4];
            int tb[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              const bool live = q + k < gs[u + 1];
              const int term = ord[live ? q + k : q];
              pr[k] = live ? (moff ? s.alpha[term] : dw_from_double(t.alpha[term])) : dw_make(0.f);
              tb[k] = term * D;
            }
            for (int d = 0; d < D; ++d) {
              if (d == j) continue;
#pragma unroll
              for (int k = 0; k < 4; ++k)
                pr[k] = dw_mul(pr[k], M[(moff ? moff[tb[k] + d] : (t.uoff[d] + t.uid[tb[k] + d]) * RR) + e]);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) acc_add(acc, pr[k]);
          }
          if (u == 0 && p.ishift != 0) {
            dw prod = eshift;
            for (int d = 0; d < D; ++d)
              if (d != j) prod = dw_mul(prod, M[(size_t)t.uoff[d] * RR + e]);
            acc_add(acc, prod);
          }
          W[(size_t)u * RR + e] = acc_value(acc);
        }
        // h_u Fo_j for every operator of mode j
        for (int item = wt; item < nu * R * nj; item += nw) {
          const int u = item / (R * nj), rem = item - u * R * nj, r = rem / nj, m = rem - r * nj;
          const int ug = t.uoff[j] + u;
          dw val;
          if (t.ident[ug]) {
            val = s.fo[r * t.nDp + opj + m];
          } else {
            const dw* h = hmat + (size_t)ug * npm * npm + (size_t)m * npm;
            dw_acc acc = acc_zero();
            for (int k = 0; k < nj; ++k) acc_fma(acc, h[k], s.fo[r * t.nDp + opj + k]);
            val = acc_value(acc);
          }
          Z[(size_t)u * R * npm + r * npm + m] = val;
        }
        asm volatile("bar.sync 2, %0;" ::"r"(nw) : "memory");
        // right-hand side b(i,n) = sum_u sum_r W_u(r,i) c_r Z_u(r,n)
        const dw* cg = pow_mode ? s.cf : s.cfo;
        for (int e = wt; e < R * nj; e += nw) {
          const int i = e % R, m = e / R;
          dw_acc acc = acc_zero();
          for (int u = 0; u < nu; ++u)
            for (int r = 0; r < R; ++r)
              acc_fma(acc, dw_mul(W[(size_t)u * RR + r * R + i], cg[r]), Z[(size_t)u * R * npm + r * npm + m]);
          const dw b = acc_value(acc);
          s.b0[i + m * R] = i >= rv ? dw_make(m == 0 ? 1.f : 0.f) : (p.ishift < 0 ? dw_neg(b) : b);
        }
      }
      __syncthreads();
      bool gj_ok = s.flags[2] != 0;
      const float* inv = s.gi + (size_t)s.flags[0] * RR;
      bool solved = false;
      const int nsw = dwsolve::solve_cols_warps(R, nj);
      if (gj_ok && R <= 32 && nj <= 16 && nsw <= kWarps) {
        if (threadIdx.x < nsw * 32) {
          const bool ok = dwsolve::solve_cols_any(s.BB, R, s.b0, s.X, nj, inv, s.cf, s.cs);
          if (threadIdx.x == 0) s.flags[3] = ok;
        }
        __syncthreads();
        solved = s.flags[3] != 0;
        gj_ok = false;  // not converged: straight to the LDL^T
      }
      if (!solved) {
        if (threadIdx.x < dwsolve::kSolverThreads) {
          int bad = 0;
          if (!(gj_ok && dwsolve::refine_solve(s.BB, R, s.b0, s.X, nj, inv, s.res, s.rred))) {
            for (int e = threadIdx.x; e < R * nj; e += dwsolve::kSolverThreads) s.X[e] = s.b0[e];
            bad = dwsolve::dw_ldlt(s.BB, R, s.dinv, s.u);
            dwsolve::dw_ldlt_solve(s.BB, R, s.dinv, s.X, nj);
          }
          dwsolve::dw_normalise_rows(s.X, R, nj, s.cf);
          if (threadIdx.x == 0 && bad) s.flags[1] = 1;
        }
        __syncthreads();
      }
      // -- the new factor: FP64 output, double-word copy and Gram (warp 0
      //    rescales the POW weights first; no other thread reads them before
      //    the next barrier) --
      if (threadIdx.x < 32) {
        for (int i = rv + threadIdx.x; i < R; i += 32) s.cf[i] = dw_make(0.f);  // ragged: padding stays weightless
        __syncwarp();
        if (pow_mode) rescale_weights_warp(s.cf, R);
        for (int i = threadIdx.x; i < R; i += 32) fc[i] = dw_to_double(s.cf[i]);
      }
      for (int e = threadIdx.x; e < R * nj; e += blockDim.x) {
        const int i = e / nj, m = e % nj;
        const dw x = s.X[i + m * R];
        fb[(size_t)i * nD + t.off[j] + m] = dw_to_double(x);
        s.f[i * t.nDp + opj + m] = x;
      }
      for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        const int i = e % R, i2 = e / R;
        if (i > i2) continue;
        dw_acc acc = acc_zero();
        for (int m = 0; m < nj; ++m) acc_fma(acc, s.X[i + m * R], s.X[i2 + m * R]);
        const dw g = acc_value(acc);
        G[(size_t)j * R * R + i + i2 * R] = g;
        G[(size_t)j * R * R + i2 + i * R] = g;
      }
      __syncthreads();
      // -- operator Grams of mode j with the new factor: h_u F_j for every
      //    operator (POW; PRODHV keeps h_u Fo_j in Z), then M_u = (h_u F_j) F_j^T --
      if (pow_mode) {
        for (int item = threadIdx.x; item < nu * R * nj; item += blockDim.x) {
          const int u = item / (R * nj), rem = item - u * R * nj, r = rem / nj, m = rem - r * nj;
          const int ug = t.uoff[j] + u;
          dw val;
          if (t.ident[ug]) {
            val = s.f[r * t.nDp + opj + m];
          } else {
            const dw* h = hmat + (size_t)ug * npm * npm + (size_t)m * npm;
            dw_acc acc = acc_zero();
            for (int k = 0; k < nj; ++k) acc_fma(acc, h[k], s.f[r * t.nDp + opj + k]);
            val = acc_value(acc);
          }
          Z[(size_t)u * R * npm + r * npm + m] = val;
        }
        __syncthreads();
      }
      for (int item = threadIdx.x; item < nu * RR; item += blockDim.x) {
        const int u = item / RR, e = item - u * RR, r = e / R, i = e - r * R;
        dw_acc acc = acc_zero();
        for (int m = 0; m < nj; ++m) acc_fma(acc, Z[(size_t)u * R * npm + r * npm + m], s.f[i * t.nDp + opj + m]);
        M[(size_t)(t.uoff[j] + u) * RR + e] = acc_value(acc);
      }
      __syncthreads();
    }
    if (pow_mode) {
      // weight renormalisation after each sweep (src/intertw_mvp.cu:491-494)
      dw part = dw_make(0.f);
      for (int e = threadIdx.x; e < R * R; e += blockDim.x) {
        dw prod = dw_mul(s.cf[e % R], s.cf[e / R]);
        for (int d = 0; d < D; ++d) prod = dw_mul(prod, G[(size_t)d * R * R + e]);
        part = dw_add(part, prod);
      }
      const dw tot = block_sum_dw(part, s.red);
      if (threadIdx.x == 0) s.misc[1] = dw_sqrt(dw_abs(tot));
      __syncthreads();
      const dw q = s.misc[1];
      for (int i = threadIdx.x; i < R; i += blockDim.x) {
        s.cf[i] = dw_div(s.cf[i], q);
        fc[i] = dw_to_double(s.cf[i]);
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0 && s.flags[1]) atomicOr(&p.status[v], 1);
}

size_t opals_smem_bytes(const OpTable& t) {
  OpSmem s;
  return carve(s, nullptr, t, true, false, false);
}

// Largest layout that fits: operators and Grams resident with the tables,
// then the tables alone, then neither (wide top-layer vectors, e.g. rank 30
// over 6 x 48 basis functions, where F and Fo take 138 KB).
int opals_launch(const OpAlsParams& p0, cudaStream_t st) {
  int dev = 0, limit = 0;
  MLCP_CUDA_TRY(cudaGetDevice(&dev));
  MLCP_CUDA_TRY(cudaDeviceGetAttribute(&limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  OpAlsParams p = p0;
  OpSmem s;
  p.tabulate = 1;
  const size_t res = carve(s, nullptr, p.ops, p.mode != 0, true, true);
  if (res <= (size_t)limit) {
    MLCP_CUDA_TRY(cudaFuncSetAttribute(opals_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)res));
    opals_kernel<true><<<p.nvec, kThreads, res, st>>>(p);
    MLCP_CUDA_TRY(cudaGetLastError());
    return kOk;
  }
  size_t smem = carve(s, nullptr, p.ops, p.mode != 0, false, true);
  if (smem > (size_t)limit) {
    p.tabulate = 0;
    smem = carve(s, nullptr, p.ops, p.mode != 0, false, false);
  }
  if (smem > (size_t)limit) {
    set_error("ALS-fitted products: rank %d over %d padded basis functions needs %zu bytes of shared memory (limit %d)",
              p.ops.R, p.ops.nDp, smem, limit);
    return kTooLarge;
  }
  MLCP_CUDA_TRY(cudaFuncSetAttribute(opals_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  opals_kernel<false><<<p.nvec, kThreads, smem, st>>>(p);
  MLCP_CUDA_TRY(cudaGetLastError());
  return kOk;
}

}  // namespace mlcp
