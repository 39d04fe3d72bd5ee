// Double-word dense kernels for one small n x n symmetric positive definite
// system, run by a team of four warps (threads 0-127 of the block) that
// synchronise on named barrier 1.  Matrices are column-major with leading
// dimension n.  Used by the ALS cluster kernel (normal equations of the rank
// reduction) and by the Gram-Schmidt kernel (normal equations of the
// orthogonalising fit).
#pragma once

#include <cfloat>

#include "dword.cuh"

namespace mlcp {
namespace dwsolve {

constexpr int kSolverWarps = 4;
constexpr int kSolverThreads = kSolverWarps * 32;

// Barrier among the solver warps only (named barrier 1).
__device__ __forceinline__ void solver_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kSolverThreads) : "memory"); }

// In-place LDL^T of the symmetric A (lower triangle): afterwards A(i,j) =
// L(i,j) for i > j and dinv[j] = 1/D(j).  The next pivot is formed first so
// its reciprocal overlaps the rest of the trailing update.  Returns the
// 1-based index of the first non-positive pivot (replaced by its magnitude
// plus a tiny amount, as the FP64 Cholesky fallback of the reference would
// fail there) or 0.  u is scratch of n entries.
__device__ inline int dw_ldlt(dw* A, int n, dw* dinv, dw* u) {
  const int t = threadIdx.x, lane = t & 31, wq = t >> 5;
  int bad = 0;
  dw d0 = A[0];
  if (!(d0.hi > 0.f)) {
    bad = 1;
    d0 = dw_make(fabsf(d0.hi) + 1e-30f);
  }
  dw inv = dw_rcp(d0);
  for (int j = 0; j < n; ++j) {
    const int m = n - j - 1;
    for (int r = t; r < m; r += kSolverThreads) {
      const dw a = A[j + 1 + r + j * n];
      u[j + 1 + r] = a;
      A[j + 1 + r + j * n] = dw_mul(a, inv);
    }
    if (t == 0) dinv[j] = inv;
    solver_sync();
    if (m == 0) break;
    dw next = dw_fms(A[j + 1 + j * n], u[j + 1], A[(j + 1) * (n + 1)]);
    if (!(next.hi > 0.f)) {
      if (!bad) bad = j + 2;
      next = dw_make(fabsf(next.hi) + 1e-30f);
    }
    const dw inv_next = dw_rcp(next);
    // trailing update: row i = j+1+ri (lane), columns j+1+cc <= i (warp-strided)
    for (int ri = lane; ri < m; ri += 32) {
      if (ri == 0) continue;  // (j+1, j+1) is `next`
      const int i = j + 1 + ri;
      const dw l = A[i + j * n];
      for (int cc = wq; cc <= ri; cc += kSolverWarps) {
        const int col = j + 1 + cc;
        A[i + col * n] = dw_fms(l, u[col], A[i + col * n]);
      }
    }
    if (t == 0) A[(j + 1) * (n + 1)] = next;
    inv = inv_next;
    solver_sync();
  }
  return bad;
}

// Solve L D L^T X = B in place for nrhs columns (B column-major, ld n).
__device__ inline void dw_ldlt_solve(const dw* A, int n, const dw* dinv, dw* B, int nrhs) {
  const int t = threadIdx.x;
  for (int j = 0; j < n - 1; ++j) {
    const int m = n - j - 1;
    for (int e = t; e < m * nrhs; e += kSolverThreads) {
      const int col = e / m, i = j + 1 + (e - col * m);
      B[i + col * n] = dw_fms(A[i + j * n], B[j + col * n], B[i + col * n]);
    }
    solver_sync();
  }
  for (int e = t; e < n * nrhs; e += kSolverThreads) {
    const int col = e / n, i = e - col * n;
    B[i + col * n] = dw_mul(B[i + col * n], dinv[i]);
  }
  solver_sync();
  for (int j = n - 1; j > 0; --j) {
    for (int e = t; e < j * nrhs; e += kSolverThreads) {
      const int col = e / j, i = e - col * j;
      B[i + col * n] = dw_fms(A[j + i * n], B[j + col * n], B[i + col * n]);
    }
    solver_sync();
  }
}

// Max-scaled 2-norm of row i of X (n entries, stride ld), as the reference's
// normonebase (src/modvecvec.cu:225-262); scales the row to unit norm.  A zero
// row gives NaN, as in the reference.
__device__ inline dw dw_normalise_row(dw* x, int n, int ld) {
  dw largest = dw_make(0.f);
  for (int q = 0; q < n; ++q) {
    const dw a = dw_abs(x[q * ld]);
    if (dw_gt(a, largest)) largest = a;
  }
  if (!(largest.hi > 0.f)) {
    const float nan = __int_as_float(0x7fffffff);
    for (int q = 0; q < n; ++q) x[q * ld] = dw_make(nan);
    return dw_make(nan);
  }
  const dw il = dw_rcp(largest);
  dw acc = dw_make(0.f);
  for (int q = 0; q < n; ++q) {
    const dw y = dw_mul(x[q * ld], il);
    acc = dw_fma(y, y, acc);
  }
  const dw r = dw_mul(largest, dw_sqrt(acc));
  const dw inv = dw_rcp(r);
  for (int q = 0; q < n; ++q) x[q * ld] = dw_mul(x[q * ld], inv);
  return r;
}

__device__ __forceinline__ dw dw_shfl_xor(dw v, int o) {
  return dw{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
}

// dw_normalise_row for all nr rows of X (column-major, ld nr, n columns) by
// the solver team, G lanes of one warp per row (G the largest power of two
// <= 32 with G nr <= 128); norms to nrm[i].  The lanes of a row combine
// their maxima and sums of squares by butterflies, so all of them hold the
// same norm.  Ends without a barrier.
__device__ inline void dw_normalise_rows(dw* X, int nr, int n, dw* nrm) {
  int G = 32;
  while (G > 1 && G * nr > kSolverThreads) G >>= 1;
  const int t = threadIdx.x, row = t / G, sub = t - row * G;
  const bool live = row < nr;
  dw* x = X + (live ? row : 0);
  dw largest = dw_make(0.f);
  for (int q = sub; q < n; q += G) {
    const dw a = dw_abs(x[q * nr]);
    if (dw_gt(a, largest)) largest = a;
  }
  for (int o = G / 2; o > 0; o >>= 1) {
    const dw b = dw_shfl_xor(largest, o);
    if (dw_gt(b, largest)) largest = b;
  }
  const bool zero = !(largest.hi > 0.f);
  const dw il = dw_rcp(zero ? dw_make(1.f) : largest);
  dw acc = dw_make(0.f);
  for (int q = sub; q < n; q += G) {
    const dw y = dw_mul(x[q * nr], il);
    acc = dw_fma(y, y, acc);
  }
  for (int o = G / 2; o > 0; o >>= 1) acc = dw_add(acc, dw_shfl_xor(acc, o));
  if (!live) return;
  if (zero) {  // NaN, as the reference's zero-row norm
    const float nan = __int_as_float(0x7fffffff);
    for (int q = sub; q < n; q += G) x[q * nr] = dw_make(nan);
    if (sub == 0) nrm[row] = dw_make(nan);
    return;
  }
  const dw r = dw_mul(largest, dw_sqrt(acc));
  const dw inv = dw_rcp(r);
  for (int q = sub; q < n; q += G) x[q * nr] = dw_mul(x[q * nr], inv);
  if (sub == 0) nrm[row] = r;
}

// Walk over the entries e = tid, tid + 128, ... of a matrix with n rows
// (column-major), tracking (row, column) = (e mod n, e div n) without dividing.
struct Walk {
  int i, j, di, dj, n;
};
__device__ __forceinline__ Walk walk_start(int t, int n) {
  return Walk{t % n, t / n, kSolverThreads % n, kSolverThreads / n, n};
}
__device__ __forceinline__ void walk_next(Walk& w) {
  w.i += w.di;
  w.j += w.dj;
  if (w.i >= w.n) {
    w.i -= w.n;
    w.j += 1;
  }
}

// Entries a solver thread handles per batch (operands loaded before any store).
constexpr int kSolveBatch = 4;

// FP32 Gauss-Jordan inverse of the symmetric positive definite n x n matrix
// given by the high parts of A (column-major), without pivoting (its pivots
// are the positive Schur-complement diagonals).  Two buffers alternate so each
// elimination step reads the previous one and needs one barrier; a thread
// loads the operands of up to four entries before it stores any (a store
// would otherwise order every later shared-memory load behind it).  Returns
// the buffer holding the inverse; *ok is false when a pivot is not positive.
__device__ inline const float* gj_inverse(const dw* A, int n, float* gi, bool* ok) {
  const int t = threadIdx.x, nn = n * n;
  for (int e = t; e < nn; e += kSolverThreads) gi[e] = A[e].hi;
  solver_sync();
  int cur = 0;
  bool good = true;
  // (row, column) of the first batch of entries, fixed for all steps
  int i0[kSolveBatch], j0[kSolveBatch];
  Walk w_later = walk_start(t, n);  // walk state at the second batch
#pragma unroll
  for (int q = 0; q < kSolveBatch; ++q) {
    i0[q] = w_later.i;
    j0[q] = w_later.j;
    walk_next(w_later);
  }
  for (int k = 0; k < n; ++k) {
    const float* s = gi + cur * nn;
    float* d = gi + (cur ^ 1) * nn;
    const float piv = s[k + k * n];
    good = good && piv > 0.f;
    float pk = f_rcp_approx(piv);
    pk = pk * fmaf(-piv, pk, 2.0f);
    Walk w = w_later;
    for (int e0 = t; e0 < nn; e0 += kSolveBatch * kSolverThreads) {
      float a[kSolveBatch], b[kSolveBatch], x[kSolveBatch];
      int ii[kSolveBatch], jj[kSolveBatch];
      const bool first = e0 == t;
#pragma unroll
      for (int q = 0; q < kSolveBatch; ++q) {
        ii[q] = first ? i0[q] : w.i;
        jj[q] = first ? j0[q] : w.j;
        if (!first) walk_next(w);
        if (e0 + q * kSolverThreads < nn) {
          a[q] = s[ii[q] + k * n];
          b[q] = s[k + jj[q] * n];
          x[q] = s[e0 + q * kSolverThreads];
        }
      }
#pragma unroll
      for (int q = 0; q < kSolveBatch; ++q) {
        const int e = e0 + q * kSolverThreads;
        if (e >= nn) continue;
        const float ta = a[q] * pk;
        float v = fmaf(-ta, b[q], x[q]);
        if (ii[q] == k) v = (jj[q] == k) ? pk : b[q] * pk;
        else if (jj[q] == k) v = -ta;
        d[e] = v;
      }
    }
    cur ^= 1;
    solver_sync();
  }
  *ok = good;
  return gi + cur * nn;
}

// The same FP32 Gauss-Jordan inverse for n <= N <= 32 by one warp, in
// registers: lane j holds column j, and each elimination step broadcasts the
// pivot column from its lane by shuffles, so no step touches shared memory or
// waits at a barrier.  Writes the inverse to inv (column-major, ld n) and
// returns whether every pivot was positive.  All 32 lanes must call it.
template <int N>
__device__ inline bool gj_inverse_warp_n(const dw* A, int n, float* inv) {
  const int lane = threadIdx.x & 31;
  const bool col = lane < n;
  float a[N];
#pragma unroll
  for (int i = 0; i < N; ++i) a[i] = (col && i < n) ? A[i + lane * n].hi : 0.f;
  bool good = true;
#pragma unroll
  for (int k = 0; k < N; ++k) {
    if (k >= n) break;
    const float piv = __shfl_sync(0xffffffffu, a[k], k);
    good = good && piv > 0.f;
    float pk = f_rcp_approx(piv);
    pk = pk * fmaf(-piv, pk, 2.0f);
    const float rk = a[k] * pk;  // row k of this column, scaled
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const float cik = __shfl_sync(0xffffffffu, a[i], k);  // column k, before the step
      if (i == k) a[i] = (lane == k) ? pk : rk;
      else a[i] = (lane == k) ? -cik * pk : fmaf(-cik, rk, a[i]);
    }
  }
  if (col)
#pragma unroll
    for (int i = 0; i < N; ++i)
      if (i < n) inv[i + lane * n] = a[i];
  return good;
}

// Register Gauss-Jordan for n <= 32, by the calling warp.
__device__ inline bool gj_inverse_warp(const dw* A, int n, float* inv) {
  if (n <= 8) return gj_inverse_warp_n<8>(A, n, inv);
  if (n <= 16) return gj_inverse_warp_n<16>(A, n, inv);
  return gj_inverse_warp_n<32>(A, n, inv);
}

// Refinement rounds before falling back to the double-word LDL^T.
constexpr int kRefineMax = 4;

// X = A^-1 B (A n x n double-word, B and X n x nrhs, ld n) by iterative
// refinement preconditioned with the FP32 inverse: X = inv B, then
// X += inv (B - A X) with the residual formed in double-word, until the last
// correction is below 1e-10 of max |X| (or the first is below 1e-5, which
// bounds the remaining error by 1e-10).  Returns whether that happened within
// kRefineMax rounds.  Each thread computes up to four entries in registers
// before storing them.
__device__ inline bool refine_solve(const dw* A, int n, const dw* B, dw* X, int nrhs, const float* inv, dw* R, float* red) {
  const int t = threadIdx.x, nr = n * nrhs;
  // X = inv * B
  {
    Walk w = walk_start(t, n);
    for (int e0 = t; e0 < nr; e0 += kSolveBatch * kSolverThreads) {
      int ii[kSolveBatch], jj[kSolveBatch];
      float acc[kSolveBatch];
#pragma unroll
      for (int q = 0; q < kSolveBatch; ++q) {
        ii[q] = w.i;
        jj[q] = w.j;
        acc[q] = 0.f;
        walk_next(w);
      }
      for (int j = 0; j < n; ++j)
#pragma unroll
        for (int q = 0; q < kSolveBatch; ++q)
          if (e0 + q * kSolverThreads < nr) acc[q] = fmaf(inv[ii[q] + j * n], B[j + jj[q] * n].hi, acc[q]);
#pragma unroll
      for (int q = 0; q < kSolveBatch; ++q)
        if (e0 + q * kSolverThreads < nr) X[e0 + q * kSolverThreads] = dw_make(acc[q]);
    }
  }
  bool ok = false;
  for (int round = 0; round < kRefineMax && !ok; ++round) {
    float* rd = red + 2 * (round & 1);
    if (t == 0) rd[0] = rd[1] = 0.f;
    solver_sync();
    // R = B - A X, compensated accumulation (two entries per thread)
    {
      Walk w = walk_start(t, n);
      for (int e0 = t; e0 < nr; e0 += 2 * kSolverThreads) {
        int ii[2], jj[2];
        dw_acc acc[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          ii[q] = w.i;
          jj[q] = w.j;
          acc[q] = acc_zero();
          if (e0 + q * kSolverThreads < nr) acc_add(acc[q], B[e0 + q * kSolverThreads]);
          walk_next(w);
        }
        const bool two = e0 + kSolverThreads < nr;
        for (int j = 0; j < n; ++j) {
          acc_fma(acc[0], dw_neg(A[ii[0] + j * n]), X[j + jj[0] * n]);
          if (two) acc_fma(acc[1], dw_neg(A[ii[1] + j * n]), X[j + jj[1] * n]);
        }
        R[e0] = acc_value(acc[0]);
        if (two) R[e0 + kSolverThreads] = acc_value(acc[1]);
      }
    }
    solver_sync();
    // X += inv * R
    float mdx = 0.f, mx = 0.f;
    {
      Walk w = walk_start(t, n);
      for (int e0 = t; e0 < nr; e0 += kSolveBatch * kSolverThreads) {
        int ii[kSolveBatch], jj[kSolveBatch];
        float acc[kSolveBatch];
        dw xv[kSolveBatch];
#pragma unroll
        for (int q = 0; q < kSolveBatch; ++q) {
          ii[q] = w.i;
          jj[q] = w.j;
          acc[q] = 0.f;
          if (e0 + q * kSolverThreads < nr) xv[q] = X[e0 + q * kSolverThreads];
          walk_next(w);
        }
        for (int j = 0; j < n; ++j)
#pragma unroll
          for (int q = 0; q < kSolveBatch; ++q)
            if (e0 + q * kSolverThreads < nr) acc[q] = fmaf(inv[ii[q] + j * n], R[j + jj[q] * n].hi, acc[q]);
#pragma unroll
        for (int q = 0; q < kSolveBatch; ++q) {
          if (e0 + q * kSolverThreads >= nr) continue;
          const dw xn = dw_add_f(xv[q], acc[q]);
          X[e0 + q * kSolverThreads] = xn;
          mdx = fmaxf(mdx, (fabsf(acc[q]) <= FLT_MAX) ? fabsf(acc[q]) : INFINITY);
          mx = fmaxf(mx, fabsf(xn.hi));
        }
      }
    }
    // non-negative floats order like their bit patterns
    atomicMax(reinterpret_cast<int*>(rd), __float_as_int(mdx));
    atomicMax(reinterpret_cast<int*>(rd + 1), __float_as_int(mx));
    solver_sync();
    // converged when the correction just applied is negligible, or when the
    // contraction it shows (rho ~ |dX|/|X|) leaves an error of rho^2 |X| <=
    // 1e-10 |X| (refinement converges linearly with rate rho), far below the
    // FP32 rounding of the right-hand side
    ok = rd[0] <= 1e-10f * rd[1] || (round == 0 && rd[0] <= 1e-5f * rd[1]);
  }
  return ok;
}


__device__ __forceinline__ dw dw_shfl(dw v, int src) {
  return dw{__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

// Shared-memory scratch of solve_cols.
struct ColScratch {
  float* conv;  // [2][32] convergence partials per warp (two rounds in flight)
  float* rmax;  // [16][32] row maxima per warp
  dw* rsum;     // [16][32] row sums of squares per warp
};

// X = A^-1 B for n <= N rows and nrhs <= 16 columns by the first
// solve_cols_warps(n, nrhs) warps of the block, synchronising on named
// barrier 3: the iterative refinement of refine_solve with the rows of the
// FP32 inverse (symmetric, so row i = column i) and of A held in registers
// and the vectors exchanged by shuffles, so that a product costs n shuffles
// and multiply-adds per lane and a round one barrier.  A warp holds H = 32/S
// columns of S >= N lanes each (column m = H w + h; lane h S + i: row i).
// When it converges, the rows of X are normalised as dw_normalise_rows does
// (norms to nrm) and it returns true; otherwise it returns false with X
// untouched.
template <int N, int S>
__device__ inline bool solve_cols(const dw* A, int n, const dw* B, dw* X, int nrhs, const float* inv, dw* nrm,
                                  const ColScratch& s) {
  constexpr int H = 32 / S;
  static_assert(N <= S && S * H == 32, "column layout");
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = lane / S, i = lane - h * S, src = h * S;
  const int m = H * w + h, nw = (nrhs + H - 1) / H, nthr = nw * 32;
  const bool row = m < nrhs && i < n;
  float iv[N];
  dw ar[N <= 16 ? N : 1];
#pragma unroll
  for (int j = 0; j < N; ++j) {
    iv[j] = (row && j < n) ? inv[i + j * n] : 0.f;
    if constexpr (N <= 16) ar[j] = (row && j < n) ? A[i + j * n] : dw_make(0.f);
  }
  const dw b = row ? B[i + m * n] : dw_make(0.f);
  float x0 = 0.f;
#pragma unroll
  for (int j = 0; j < N; ++j) x0 = fmaf(iv[j], __shfl_sync(0xffffffffu, b.hi, src + j), x0);
  dw x = dw_make(x0);
  bool ok = false;
  for (int round = 0; round < kRefineMax && !ok; ++round) {
    // r = b - A x (compensated), then the FP32 correction inv r
    dw_acc acc = acc_zero();
    acc_add(acc, b);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      const dw xj = dw_shfl(x, src + j);
      dw aij;
      if constexpr (N <= 16) aij = ar[j];
      else aij = (row && j < n) ? A[i + j * n] : dw_make(0.f);
      acc_fma(acc, dw_neg(aij), xj);
    }
    const dw r = acc_value(acc);
    float d = 0.f;
#pragma unroll
    for (int j = 0; j < N; ++j) d = fmaf(iv[j], __shfl_sync(0xffffffffu, r.hi, src + j), d);
    if (row) x = dw_add_f(x, d);
    float mdx = row ? ((fabsf(d) <= FLT_MAX) ? fabsf(d) : INFINITY) : 0.f;
    float mx = row ? fabsf(x.hi) : 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      mdx = fmaxf(mdx, __shfl_xor_sync(0xffffffffu, mdx, o));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    float* cv = s.conv + (round & 1) * 32;
    if (lane == 0) {
      cv[w] = mdx;
      cv[16 + w] = mx;
    }
    asm volatile("bar.sync 3, %0;" ::"r"(nthr) : "memory");
    float gd = 0.f, gx = 0.f;
    for (int q = 0; q < nw; ++q) {
      gd = fmaxf(gd, cv[q]);
      gx = fmaxf(gx, cv[16 + q]);
    }
    // the convergence rule of refine_solve
    ok = gd <= 1e-10f * gx || (round == 0 && gd <= 1e-5f * gx);
  }
  if (!ok) return false;
  // rows: scale by the largest |x|, sum the squares over the columns
  const int slot = (m < 16 ? m : 15) * 32 + i;
  if (m < nrhs) s.rmax[slot] = fabsf(x.hi);
  asm volatile("bar.sync 3, %0;" ::"r"(nthr) : "memory");
  float big = 0.f;
  for (int q = 0; q < nrhs; ++q) big = fmaxf(big, s.rmax[q * 32 + i]);
  const bool zero = !(big > 0.f);
  const dw il = dw_rcp(dw_make(zero ? 1.f : big));
  const dw y = dw_mul(x, il);
  if (m < nrhs) s.rsum[slot] = dw_mul(y, y);
  asm volatile("bar.sync 3, %0;" ::"r"(nthr) : "memory");
  dw_acc sq = acc_zero();
  for (int q = 0; q < nrhs; ++q) acc_add(sq, s.rsum[q * 32 + i]);
  if (!row) return true;
  if (zero) {  // NaN, as the reference's zero-row norm
    const float nan = __int_as_float(0x7fffffff);
    X[i + m * n] = dw_make(nan);
    if (m == 0) nrm[i] = dw_make(nan);
    return true;
  }
  const dw r = dw_mul(dw_make(big), dw_sqrt(acc_value(sq)));
  X[i + m * n] = dw_mul(x, dw_rcp(r));
  if (m == 0) nrm[i] = r;
  return true;
}

// Warps used by solve_cols_any for an n-row system with nrhs columns.
__host__ __device__ inline int solve_cols_warps(int n, int nrhs) { return n <= 16 ? (nrhs + 1) / 2 : nrhs; }

// solve_cols for n <= 32 (two columns per warp when n <= 16).
__device__ inline bool solve_cols_any(const dw* A, int n, const dw* B, dw* X, int nrhs, const float* inv, dw* nrm,
                                      const ColScratch& s) {
  if (n <= 16) return solve_cols<16, 16>(A, n, B, X, nrhs, inv, nrm, s);
  return solve_cols<32, 32>(A, n, B, X, nrhs, inv, nrm, s);
}

// solve_cols for n <= 16 with one column per warp and each row's sums split
// over the two half-warps (lane h 16 + i: row i, terms j of half h), so that
// every dependency chain is half as long; the halves combine their partial
// results in a fixed order, so both hold identical values.  Uses warps
// 0..nrhs-1 (named barrier 3); same results contract as solve_cols.
__device__ __forceinline__ dw_acc acc_merge(dw_acc a, dw_acc b) {
  const dw t = two_sum(a.s, b.s);
  return dw_acc{t.hi, f_add(f_add(a.c, b.c), t.lo)};
}
__device__ inline bool solve_cols_split(const dw* A, int n, const dw* B, dw* X, int nrhs, const float* inv, dw* nrm,
                                        const ColScratch& s) {
  constexpr int NH = 8;
  const int lane = threadIdx.x & 31, m = threadIdx.x >> 5, i = lane & 15, h = lane >> 4, j0 = h * NH;
  const int nthr = nrhs * 32;
  const bool row = i < n;
  float iv[NH];
  dw ar[NH];
#pragma unroll
  for (int q = 0; q < NH; ++q) {
    const int j = j0 + q;
    iv[q] = (row && j < n) ? inv[i + j * n] : 0.f;
    ar[q] = (row && j < n) ? A[i + j * n] : dw_make(0.f);
  }
  const dw b = row ? B[i + m * n] : dw_make(0.f);
  auto combine = [&](float v) {  // fixed order: half 0's part first
    const float o = __shfl_xor_sync(0xffffffffu, v, 16);
    return h == 0 ? v + o : o + v;
  };
  float p0 = 0.f;
#pragma unroll
  for (int q = 0; q < NH; ++q) p0 = fmaf(iv[q], __shfl_sync(0xffffffffu, b.hi, j0 + q), p0);
  dw x = dw_make(combine(p0));
  bool ok = false;
  for (int round = 0; round < kRefineMax && !ok; ++round) {
    dw_acc acc = acc_zero();
    if (h == 0) acc_add(acc, b);
#pragma unroll
    for (int q = 0; q < NH; ++q) acc_fma(acc, dw_neg(ar[q]), dw_shfl(x, j0 + q));
    const dw_acc other{__shfl_xor_sync(0xffffffffu, acc.s, 16), __shfl_xor_sync(0xffffffffu, acc.c, 16)};
    const dw r = acc_value(h == 0 ? acc_merge(acc, other) : acc_merge(other, acc));
    float dp = 0.f;
#pragma unroll
    for (int q = 0; q < NH; ++q) dp = fmaf(iv[q], __shfl_sync(0xffffffffu, r.hi, j0 + q), dp);
    const float d = combine(dp);
    if (row) x = dw_add_f(x, d);
    float mdx = row ? ((fabsf(d) <= FLT_MAX) ? fabsf(d) : INFINITY) : 0.f;
    float mx = row ? fabsf(x.hi) : 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      mdx = fmaxf(mdx, __shfl_xor_sync(0xffffffffu, mdx, o));
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    }
    float* cv = s.conv + (round & 1) * 32;
    if (lane == 0) {
      cv[m] = mdx;
      cv[16 + m] = mx;
    }
    asm volatile("bar.sync 3, %0;" ::"r"(nthr) : "memory");
    float gd = 0.f, gx = 0.f;
    for (int w = 0; w < nrhs; ++w) {
      gd = fmaxf(gd, cv[w]);
      gx = fmaxf(gx, cv[16 + w]);
    }
    ok = gd <= 1e-10f * gx || (round == 0 && gd <= 1e-5f * gx);
  }
  if (!ok) return false;
  const int slot = m * 32 + i;
  if (h == 0) s.rmax[slot] = fabsf(x.hi);
  asm volatile("bar.sync 3, %0;" ::"r"(nthr) : "memory");
  float big = 0.f;
  for (int w = 0; w < nrhs; ++w) big = fmaxf(big, s.rmax[w * 32 + i]);
  const bool zero = !(big > 0.f);
  const dw il = dw_rcp(dw_make(zero ? 1.f : big));
  const dw y = dw_mul(x, il);
  if (h == 0) s.rsum[slot] = dw_mul(y, y);
  asm volatile("bar.sync 3, %0;" ::"r"(nthr) : "memory");
  dw_acc sq = acc_zero();
  for (int w = 0; w < nrhs; ++w) acc_add(sq, s.rsum[w * 32 + i]);
  if (!row || h != 0) return true;
  if (zero) {  // NaN, as the reference's zero-row norm
    const float nan = __int_as_float(0x7fffffff);
    X[i + m * n] = dw_make(nan);
    if (m == 0) nrm[i] = dw_make(nan);
    return true;
  }
  const dw rn = dw_mul(dw_make(big), dw_sqrt(acc_value(sq)));
  X[i + m * n] = dw_mul(x, dw_rcp(rn));
  if (m == 0) nrm[i] = rn;
  return true;
}

}  // namespace dwsolve
}  // namespace mlcp
