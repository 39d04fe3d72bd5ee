// Shared helpers for the GB300 CP-format hot path.
//
// CP-vector layout (reference src/cpvector.cu:407-414): term r, mode d,
// index i at base[r*nD + off[d] + i], one weight coef[r] per term.  Every
// kernel here reads and writes that layout for caller-visible data; private
// working copies (FP32 factors, mode-major target factors) are described
// where they are built.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstdarg>
#include <string>

namespace mlcp {

// Last error message of the calling host thread (queried through
// mlcp_gb300_last_error()).  Entry points never exit the process.
void set_error(const char* fmt, ...);
const char* last_error();

// Error codes returned by the C entry points.
enum Status : int {
  kOk = 0,
  kBadArgument = 1,
  kTooLarge = 2,
  kCudaError = 3,
  kNumerical = 4,
};


}  // namespace mlcp

#define MLCP_CUDA_TRY(expr)                                                              \
  do {                                                                                   \
    cudaError_t err__ = (expr);                                                          \
    if (err__ != cudaSuccess) {                                                          \
      mlcp::set_error("%s failed at %s:%d: %s", #expr, __FILE__, __LINE__,               \
                      cudaGetErrorString(err__));                                        \
      return mlcp::kCudaError;                                                           \
    }                                                                                    \
  } while (0)

namespace mlcp {

__host__ __device__ inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// ---------------------------------------------------------------------------
// FP64 dense kernels for one R x R system, executed by one thread block.
// All matrices are column-major in shared memory with leading dimension ld.
// ---------------------------------------------------------------------------

// In-place Cholesky A = L L^T of the lower triangle (upper part untouched).
// Returns through *info the first non-positive pivot (1-based) or 0.
__device__ inline void block_cholesky(double* A, int n, int ld, int* info) {
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) *info = 0;
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (tid == 0) {
      double d = A[j + j * ld];
      if (!(d > 0.0)) {
        if (*info == 0) *info = j + 1;
        d = fabs(d) + 1e-300;
      }
      A[j + j * ld] = sqrt(d);
    }
    __syncthreads();
    const double ljj = A[j + j * ld];
    for (int i = j + 1 + tid; i < n; i += nt) A[i + j * ld] /= ljj;
    __syncthreads();
    // trailing update of the lower triangle: columns c in (j, n), rows i >= c
    const int m = n - j - 1;
    const int ntri = m * (m + 1) / 2;
    for (int e = tid; e < ntri; e += nt) {
      // map e -> (c, i) with c = j+1+cc, i = c + ii
      int cc = 0, rem = e, len = m;
      while (rem >= len) { rem -= len; --len; ++cc; }
      const int c = j + 1 + cc, i = c + rem;
      A[i + c * ld] -= A[i + j * ld] * A[c + j * ld];
    }
    __syncthreads();
  }
}

// Solve L L^T X = B for nrhs columns (B column-major, leading dim ldb),
// parallel over right-hand sides.
__device__ inline void block_cholesky_solve(const double* L, int n, int ld, double* B, int nrhs, int ldb) {
  for (int c = threadIdx.x; c < nrhs; c += blockDim.x) {
    double* b = B + c * ldb;
    for (int j = 0; j < n; ++j) {
      double t = b[j];
      for (int k = 0; k < j; ++k) t -= L[j + k * ld] * b[k];
      b[j] = t / L[j + j * ld];
    }
    for (int j = n - 1; j >= 0; --j) {
      double t = b[j];
      for (int k = j + 1; k < n; ++k) t -= L[k + j * ld] * b[k];
      b[j] = t / L[j + j * ld];
    }
  }
  __syncthreads();
}


// ---------------------------------------------------------------------------
// Latency-lean FP64 kernels.  On this GPU a dependent FP64 operation costs
// ~64 cycles, FP64 division/square root ~650 cycles, and the FP64 pipe issues
// two lanes per cycle per SM.  So: pivots use reciprocals from an FP32 seed
// refined by Newton-Raphson in FP64 (no FP64 division or square root on a
// critical path), the factorisation is LDL^T (no square root), and the small
// dense kernels run on one warp so that redundant copies of the same
// operation do not occupy the FP64 pipe.
// ---------------------------------------------------------------------------

// 1/d from an FP32 seed (about 23 correct bits) and one FP64 Newton step
// (about 46 bits); `full` adds a second step (full precision).
__device__ __forceinline__ double rcp64(double d, bool full = true) {
  float seed;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(seed) : "f"((float)d));
  double r = (double)seed;
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  if (full) {
    e = fma(-d, r, 1.0);
    r = fma(r, e, r);
  }
  return r;
}

// 1/sqrt(d) from an FP32 seed and two FP64 Newton steps.
__device__ __forceinline__ double rsqrt64(double d) {
  double y = (double)rsqrtf((float)d);
  const double h = 0.5 * d;
  y = y * fma(-h * y, y, 1.5);
  return y * fma(-h * y, y, 1.5);
}

// Threads that run the small FP64 kernels: four warps, one per SM
// sub-partition (each sub-partition's FP64 unit retires half a lane per
// cycle, so a 32-lane FP64 instruction costs it ~64 cycles).
constexpr int kFp64Threads = 128;

// Barrier among the first kFp64Threads threads only (named barrier 1).
__device__ __forceinline__ void fp64_sync() { asm volatile("bar.sync 1, %0;" ::"r"(kFp64Threads) : "memory"); }

// In-place LDL^T of the symmetric n x n matrix A (lower triangle used), run by
// the first kFp64Threads threads: afterwards A(i,j) = L(i,j) for i > j and
// dinv[j] = 1 / D(j) (46-bit reciprocal, far below the FP32-level noise of the
// right-hand sides).  The next pivot is updated first so that its reciprocal
// overlaps the rest of the trailing update.  u is scratch of n doubles.
// Call from all threads of the block.
__device__ inline void block_ldlt(double* A, int n, int ld, double* dinv, double* u, int* info) {
  __syncthreads();
  const int t = threadIdx.x;
  if (t < kFp64Threads) {
    int bad = 0;
    double d0 = A[0];
    if (!(d0 > 0.0)) { bad = 1; d0 = fabs(d0) + 1e-300; }
    double inv = rcp64(d0, false);
    for (int j = 0; j < n; ++j) {
      const int m = n - j - 1;
      // column j: keep the unscaled values (u), store L(i,j)
      if (t < m) {
        const double a = A[j + 1 + t + j * ld];
        u[j + 1 + t] = a;
        A[j + 1 + t + j * ld] = a * inv;
      }
      if (t == 0) dinv[j] = inv;
      fp64_sync();
      if (m == 0) break;
      // next pivot first
      double next = fma(-A[j + 1 + j * ld], u[j + 1], A[j + 1 + (j + 1) * ld]);
      if (!(next > 0.0)) {
        if (bad == 0) bad = j + 2;
        next = fabs(next) + 1e-300;
      }
      const double inv_next = rcp64(next, false);
      // rest of the trailing update: pairs (i, c), j+1 <= c <= i < n, minus (j+1, j+1)
      const int ntri = m * (m + 1) / 2;
      for (int e = 1 + t; e < ntri; e += kFp64Threads) {
        // packed column-major index e -> (cc, ii), 0 <= cc <= ii < m
        int cc = (int)((2.f * m + 1.f - sqrtf((2.f * m + 1.f) * (2.f * m + 1.f) - 8.f * e)) * 0.5f);
        cc = max(0, min(cc, m - 1));
        while (cc > 0 && cc * (2 * m - cc + 1) / 2 > e) --cc;
        while ((cc + 1) * (2 * m - cc) / 2 <= e) ++cc;
        const int c = j + 1 + cc, i = c + (e - cc * (2 * m - cc + 1) / 2);
        const double l = A[i + j * ld], uc = u[c], a = A[i + c * ld];
        A[i + c * ld] = fma(-l, uc, a);
      }
      if (t == 0) A[j + 1 + (j + 1) * ld] = next;
      inv = inv_next;
      fp64_sync();
    }
    if (t == 0) *info = bad;
  }
  __syncthreads();
}

// Max-scaled 2-norm of x[0], x[stride], ..., x[(n-1)*stride] (reference
// normonebase, src/modvecvec.cu:225-262) and its reciprocal.
__device__ inline void scaled_norm(const double* x, int n, int stride, double* nrm, double* inv) {
  double largest = 0.0;
  for (int q = 0; q < n; ++q) largest = fmax(largest, fabs(x[q * stride]));
  const double il = rcp64(largest);
  double acc = 0.0;
  for (int q = 0; q < n; ++q) {
    const double t = x[q * stride] * il;
    acc = fma(t, t, acc);
  }
  // acc >= 1 whenever largest > 0; a zero factor gives NaN as in the reference
  const double r = largest * (acc * rsqrt64(acc));
  *nrm = (largest > 0.0) ? r : largest / largest;
  *inv = rcp64(*nrm);
}

// Solve L D L^T X = B for nrhs columns with the factor from block_ldlt, run by
// the first kFp64Threads threads; each elimination step spreads the
// (row, column) pairs of all right-hand sides over the four warps.
__device__ inline void block_ldlt_solve(const double* A, int n, int ld, const double* dinv, double* B, int nrhs,
                                        int ldb) {
  __syncthreads();
  const int t = threadIdx.x;
  if (t < kFp64Threads) {
    for (int j = 0; j < n - 1; ++j) {  // forward: unit lower L
      const int m = n - j - 1;
      for (int e = t; e < m * nrhs; e += kFp64Threads) {
        const int c = e / m, i = j + 1 + (e - c * m);
        const double l = A[i + j * ld], bj = B[j + c * ldb], bi = B[i + c * ldb];
        B[i + c * ldb] = fma(-l, bj, bi);
      }
      fp64_sync();
    }
    for (int e = t; e < n * nrhs; e += kFp64Threads) {
      const int c = e / n, i = e - c * n;
      B[i + c * ldb] *= dinv[i];
    }
    fp64_sync();
    for (int j = n - 1; j > 0; --j) {  // backward: L^T
      for (int e = t; e < j * nrhs; e += kFp64Threads) {
        const int c = e / j, i = e - c * j;
        const double l = A[j + i * ld], bj = B[j + c * ldb], bi = B[i + c * ldb];
        B[i + c * ldb] = fma(-l, bj, bi);
      }
      fp64_sync();
    }
  }
  __syncthreads();
}

}  // namespace mlcp
