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

}  // namespace mlcp
