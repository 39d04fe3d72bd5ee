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

}  // namespace mlcp
