// Division by a run-time invariant divisor as a multiply-high and two shifts.
//
// The kernels split flat work indices e into (row, column) pairs by divisors
// that are fixed for a launch (ranks, basis sizes) but not known at compile
// time; a generic 32-bit integer division costs a few dozen instructions.
// FastDiv precomputes the magic multiplier of Granlund and Montgomery
// ("Division by invariant integers using multiplication", PLDI 1994,
// Figure 4.1, the unsigned round-up method): with l = ceil(log2 d) and
// m = floor(2^32 (2^l - d) / d) + 1,
//   q = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0),   t = mulhi(m, n),
// which equals floor(n / d) for every 32-bit unsigned n and 1 <= d < 2^31.
// tests/test_fastdiv.py compiles this header on the host and checks it
// against the plain division.
#pragma once

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

namespace mlcp {

struct FastDiv {
  unsigned d = 1, m = 1;
  int s1 = 0, s2 = 0;

  FastDiv() = default;
  __host__ __device__ explicit FastDiv(unsigned dv) : d(dv) {
    int l = 0;
    while ((1ull << l) < (unsigned long long)dv) ++l;
    m = (unsigned)((((1ull << l) - dv) << 32) / dv + 1ull);
    s1 = l > 0 ? 1 : 0;
    s2 = l > 0 ? l - 1 : 0;
  }
  __host__ __device__ __forceinline__ unsigned div(unsigned n) const {
#ifdef __CUDA_ARCH__
    const unsigned t = __umulhi(m, n);
#else
    const unsigned t = (unsigned)(((unsigned long long)m * n) >> 32);
#endif
    return (t + ((n - t) >> s1)) >> s2;
  }
  // n = q d + r with 0 <= r < d
  __host__ __device__ __forceinline__ void divmod(unsigned n, int* q, int* r) const {
    const unsigned qq = div(n);
    *q = (int)qq;
    *r = (int)(n - qq * d);
  }
};

}  // namespace mlcp
