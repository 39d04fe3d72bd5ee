// Double-word ("float-float") arithmetic: a value is hi + lo with two FP32
// numbers, |lo| <= ulp(hi)/2, carrying about 48 significant bits.
//
// Why: on GB300 an FP64 instruction occupies the SM's FP64 pipe for 64 cycles
// per warp whatever its active-lane count, and the pipe is shared by the SM
// (measured: 16 warps each running a dependent FP64 FMA chain advance one
// operation per 304 cycles).  A double-word FMA runs on the FP32 pipes in
// ~36 cycles of dependent latency with 128 lanes per cycle of throughput, so
// the small dense solves of the ALS step run faster in double-word than in
// FP64 and leave the FP64 pipe alone.  48 bits is far beyond what the solves
// need: their right-hand sides are FP32 contractions (24 bits).
//
// Algorithms (published, restated here):
//   TwoSum            Knuth, TAOCP vol. 2 (1969), 4.2.2 Theorem B
//   Fast2Sum          Dekker, Numer. Math. 18 (1971) 224-242
//   TwoProd (FMA)     exact product error by one fused multiply-add
//   DWPlusDW          Joldes, Muller, Popescu, ACM TOMS 44(2) 2017, Alg. 6
//                     ("AccurateDWPlusDW", relative error <= 3u^2 + 13u^3),
//                     and Alg. 5 ("SloppyDWPlusDW") for residual sums
//   DWTimesDW         same paper, Alg. 12 (relative error <= 5u^2)
//   reciprocal, sqrt  one Newton-Raphson step in double-word from an FP32
//                     approximation (quadratic convergence: 2^-23 -> 2^-46)
// Every FP32 operation is written with explicit rounding intrinsics on the
// device so the compiler cannot contract a multiply and an add of these
// error-free transformations into one FMA.  Host builds must use
// -ffp-contract=off (the CPU tests compile this header that way).
#pragma once

#include <cmath>
#include <cfloat>

#ifdef __CUDACC__
#define MLCP_HD __host__ __device__ __forceinline__
#else
#define MLCP_HD inline
#endif

namespace mlcp {

struct dw {
  float hi, lo;
};

#if defined(__CUDA_ARCH__)
MLCP_HD float f_add(float a, float b) { return __fadd_rn(a, b); }
MLCP_HD float f_sub(float a, float b) { return __fsub_rn(a, b); }
MLCP_HD float f_mul(float a, float b) { return __fmul_rn(a, b); }
MLCP_HD float f_fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
// FP32 approximations used as Newton seeds (relative error below 2^-22).
MLCP_HD float f_rcp_approx(float a) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}
MLCP_HD float f_rsqrt_approx(float a) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(a));
  return r;
}
#else
MLCP_HD float f_add(float a, float b) { return a + b; }
MLCP_HD float f_sub(float a, float b) { return a - b; }
MLCP_HD float f_mul(float a, float b) { return a * b; }
MLCP_HD float f_fma(float a, float b, float c) { return std::fma(a, b, c); }
MLCP_HD float f_rcp_approx(float a) { return 1.0f / a; }
MLCP_HD float f_rsqrt_approx(float a) { return 1.0f / std::sqrt(a); }
#endif

MLCP_HD dw dw_make(float hi, float lo = 0.f) { return dw{hi, lo}; }

// s + e = a + b exactly (any a, b).
MLCP_HD dw two_sum(float a, float b) {
  const float s = f_add(a, b);
  const float bb = f_sub(s, a);
  const float e = f_add(f_sub(a, f_sub(s, bb)), f_sub(b, bb));
  return dw{s, e};
}

// s + e = a + b exactly when |a| >= |b| (or a == 0).
MLCP_HD dw fast_two_sum(float a, float b) {
  const float s = f_add(a, b);
  return dw{s, f_sub(b, f_sub(s, a))};
}

// p + e = a * b exactly (barring underflow).
MLCP_HD dw two_prod(float a, float b) {
  const float p = f_mul(a, b);
  return dw{p, f_fma(a, b, -p)};
}

MLCP_HD dw dw_add(dw x, dw y) {
  const dw s = two_sum(x.hi, y.hi);
  const dw t = two_sum(x.lo, y.lo);
  const float c = f_add(s.lo, t.hi);
  const dw v = fast_two_sum(s.hi, c);
  const float w = f_add(t.lo, v.lo);
  return fast_two_sum(v.hi, w);
}

// x + y with JMP17 Alg. 5 ("SloppyDWPlusDW"): the error is bounded by about
// u^2 (|x| + |y|) rather than relative to the sum, which is what accumulations
// of residuals need, for about half the operations of dw_add.
MLCP_HD dw dw_add_sloppy(dw x, dw y) {
  const dw s = two_sum(x.hi, y.hi);
  const float v = f_add(x.lo, y.lo);
  const float w = f_add(s.lo, v);
  return fast_two_sum(s.hi, w);
}

MLCP_HD dw dw_neg(dw x) { return dw{-x.hi, -x.lo}; }
MLCP_HD dw dw_sub(dw x, dw y) { return dw_add(x, dw_neg(y)); }

// x + b for an FP32 b (JMP17 Alg. 4, DWPlusFP).
MLCP_HD dw dw_add_f(dw x, float b) {
  const dw s = two_sum(x.hi, b);
  const float v = f_add(x.lo, s.lo);
  return fast_two_sum(s.hi, v);
}

MLCP_HD dw dw_mul(dw x, dw y) {
  const dw c = two_prod(x.hi, y.hi);
  const float tl0 = f_mul(x.lo, y.lo);
  const float tl1 = f_fma(x.hi, y.lo, tl0);
  const float cl2 = f_fma(x.lo, y.hi, tl1);
  const float cl3 = f_add(c.lo, cl2);
  return fast_two_sum(c.hi, cl3);
}

// x * b for an FP32 b (JMP17 Alg. 9, DWTimesFP3).
MLCP_HD dw dw_mul_f(dw x, float b) {
  const dw c = two_prod(x.hi, b);
  const float cl3 = f_fma(x.lo, b, c.lo);
  return fast_two_sum(c.hi, cl3);
}

// z + x * y
MLCP_HD dw dw_fma(dw x, dw y, dw z) { return dw_add(z, dw_mul(x, y)); }
// z - x * y
MLCP_HD dw dw_fms(dw x, dw y, dw z) { return dw_sub(z, dw_mul(x, y)); }

// 1 / a: FP32 seed r0, residual e = 1 - a r0 formed exactly enough
// (1 - hi*r0 is exact by Sterbenz once the product's error term is split
// off), then r0 + r0 e.
MLCP_HD dw dw_rcp(dw a) {
  const float r0 = f_rcp_approx(a.hi);
  const dw p = two_prod(a.hi, r0);
  float e = f_sub(f_sub(1.0f, p.hi), p.lo);
  e = f_fma(-a.lo, r0, e);
  return fast_two_sum(r0, f_mul(r0, e));
}

// b / a
MLCP_HD dw dw_div(dw b, dw a) { return dw_mul(b, dw_rcp(a)); }

// sqrt(a) for a > 0: s0 = a y0 with y0 ~ a^-1/2, then s0 + y0 (a - s0^2) / 2.
MLCP_HD dw dw_sqrt(dw a) {
  if (!(a.hi > 0.f)) return dw{0.f, 0.f};
  const float y0 = f_rsqrt_approx(a.hi);
  const float s0 = f_mul(a.hi, y0);
  const dw p = two_prod(s0, s0);
  const float r = f_add(f_sub(f_sub(a.hi, p.hi), p.lo), a.lo);
  return fast_two_sum(s0, f_mul(f_mul(0.5f, y0), r));
}

// Compensated accumulation of a sum of products of double-word values: the
// FP32 running sum s and, in c, the FP32 sum of the exact errors of each
// product (two_prod) and addition (two_sum) together with the products'
// low-order cross terms.  This is the dot product Dot2 of Ogita, Rump and
// Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005)
// with double-word operands.  Its error is about n u^2 sum |x_i y_i|, as for
// a chain of dw_fma, but the dependency chain through s is one FP32 addition
// per term and a term costs about half the instructions.
struct dw_acc {
  float s, c;
};
MLCP_HD dw_acc acc_zero() { return dw_acc{0.f, 0.f}; }
MLCP_HD void acc_fma(dw_acc& a, dw x, dw y) {
  const dw p = two_prod(x.hi, y.hi);
  const dw t = two_sum(a.s, p.hi);
  a.s = t.hi;
  a.c = f_add(a.c, f_add(f_add(t.lo, p.lo), f_fma(x.hi, y.lo, f_mul(x.lo, y.hi))));
}
MLCP_HD void acc_add(dw_acc& a, dw x) {
  const dw t = two_sum(a.s, x.hi);
  a.s = t.hi;
  a.c = f_add(a.c, f_add(t.lo, x.lo));
}
MLCP_HD dw acc_value(dw_acc a) { return two_sum(a.s, a.c); }

MLCP_HD dw dw_abs(dw a) { return (a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f)) ? dw_neg(a) : a; }
MLCP_HD bool dw_gt(dw a, dw b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }

// Conversions to and from FP64 (these three use the FP64 pipe; keep them
// off the critical paths).
MLCP_HD dw dw_from_double(double x) {
  const float hi = (float)x;
  return dw{hi, (float)(x - (double)hi)};
}
MLCP_HD double dw_to_double(dw a) { return (double)a.hi + (double)a.lo; }

}  // namespace mlcp
