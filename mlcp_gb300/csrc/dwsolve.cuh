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
    // R = B - A X (double-word); two chains per entry (even and odd j)
    {
      Walk w = walk_start(t, n);
      for (int e0 = t; e0 < nr; e0 += 2 * kSolverThreads) {
        int ii[2], jj[2];
        dw a0[2], a1[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          ii[q] = w.i;
          jj[q] = w.j;
          a0[q] = (e0 + q * kSolverThreads < nr) ? B[e0 + q * kSolverThreads] : dw_make(0.f);
          a1[q] = dw_make(0.f);
          walk_next(w);
        }
        const bool two = e0 + kSolverThreads < nr;
        int j = 0;
        for (; j + 1 < n; j += 2) {
          a0[0] = dw_add_sloppy(a0[0], dw_neg(dw_mul(A[ii[0] + j * n], X[j + jj[0] * n])));
          a1[0] = dw_add_sloppy(a1[0], dw_neg(dw_mul(A[ii[0] + (j + 1) * n], X[j + 1 + jj[0] * n])));
          if (two) {
            a0[1] = dw_add_sloppy(a0[1], dw_neg(dw_mul(A[ii[1] + j * n], X[j + jj[1] * n])));
            a1[1] = dw_add_sloppy(a1[1], dw_neg(dw_mul(A[ii[1] + (j + 1) * n], X[j + 1 + jj[1] * n])));
          }
        }
        if (j < n) {
          a0[0] = dw_add_sloppy(a0[0], dw_neg(dw_mul(A[ii[0] + j * n], X[j + jj[0] * n])));
          if (two) a0[1] = dw_add_sloppy(a0[1], dw_neg(dw_mul(A[ii[1] + j * n], X[j + jj[1] * n])));
        }
        R[e0] = dw_add_sloppy(a0[0], a1[0]);
        if (two) R[e0 + kSolverThreads] = dw_add_sloppy(a0[1], a1[1]);
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

}  // namespace dwsolve
}  // namespace mlcp
