// Accuracy check of the double-word arithmetic in mlcp_gb300/csrc/dword.cuh
// against long double, on seeded random operands.  Prints one line per
// operation: "<name> <max relative error as -log2>".
// Build: g++ -O2 -ffp-contract=off -I mlcp_gb300/csrc dword_check.cpp
#include <cmath>
#include <cstdint>
#include <cstdio>

#include "dword.cuh"

using mlcp::dw;

static uint64_t g_state = 0x9E3779B97F4A7C15ull;
static double uniform() {  // splitmix64 -> [0, 1)
  uint64_t z = (g_state += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

// A random double-word value with magnitude spread over [2^-e, 2^e).
static dw random_dw(int e, bool positive) {
  const double mant = 1.0 + uniform();
  const double ex = std::ldexp(1.0, (int)std::floor((uniform() * 2.0 - 1.0) * e));
  double x = mant * ex;
  if (!positive && uniform() < 0.5) x = -x;
  return mlcp::dw_from_double(x);
}

static long double ld(dw a) { return (long double)a.hi + (long double)a.lo; }

static double relerr(long double got, long double want) {
  if (want == 0.0L) return (double)fabsl(got);
  return (double)fabsl((got - want) / want);
}

static double scaled(long double got, long double want, long double mag) {
  return (double)(fabsl(got - want) / mag);
}

static void report(const char* name, double worst) {
  std::printf("%s %.2f\n", name, worst > 0 ? -std::log2(worst) : 99.0);
}

int main() {
  const int n = 200000;
  double e_adds = 0, e_add = 0, e_mul = 0, e_fma = 0, e_rcp = 0, e_div = 0, e_sqrt = 0, e_addf = 0, e_mulf = 0, e_conv = 0;
  for (int t = 0; t < n; ++t) {
    const dw a = random_dw(20, false), b = random_dw(20, false), c = random_dw(20, false);
    const dw p = random_dw(20, true);
    // sums: error relative to the operand magnitudes (|a| + |b|), the form in
    // which the bounds are stated; cancellation is then no concern
    e_add = std::fmax(e_add, scaled(ld(mlcp::dw_add(a, b)), ld(a) + ld(b), fabsl(ld(a)) + fabsl(ld(b))));
    e_adds = std::fmax(e_adds, scaled(ld(mlcp::dw_add_sloppy(a, b)), ld(a) + ld(b), fabsl(ld(a)) + fabsl(ld(b))));
    e_mul = std::fmax(e_mul, relerr(ld(mlcp::dw_mul(a, b)), ld(a) * ld(b)));
    const long double fw = ld(a) * ld(b) + ld(c);
    e_fma = std::fmax(e_fma, scaled(ld(mlcp::dw_fma(a, b, c)), fw, fabsl(ld(a) * ld(b)) + fabsl(ld(c))));
    e_rcp = std::fmax(e_rcp, relerr(ld(mlcp::dw_rcp(a)), 1.0L / ld(a)));
    e_div = std::fmax(e_div, relerr(ld(mlcp::dw_div(b, a)), ld(b) / ld(a)));
    e_sqrt = std::fmax(e_sqrt, relerr(ld(mlcp::dw_sqrt(p)), sqrtl(ld(p))));
    const float f = b.hi;
    e_addf = std::fmax(e_addf, scaled(ld(mlcp::dw_add_f(a, f)), ld(a) + (long double)f,
                                      fabsl(ld(a)) + fabsl((long double)f)));
    e_mulf = std::fmax(e_mulf, relerr(ld(mlcp::dw_mul_f(a, f)), ld(a) * (long double)f));
    const double x = (1.0 + uniform()) * std::ldexp(1.0, (int)(uniform() * 40) - 20);
    e_conv = std::fmax(e_conv, relerr(ld(mlcp::dw_from_double(x)), (long double)x));
  }
  report("add", e_add);
  report("add_sloppy", e_adds);
  report("mul", e_mul);
  report("fma", e_fma);
  report("rcp", e_rcp);
  report("div", e_div);
  report("sqrt", e_sqrt);
  // compensated dot products of 1..40 terms: error relative to sum |x_i y_i|
  double e_dot = 0, e_sum = 0;
  for (int t = 0; t < 20000; ++t) {
    const int nt = 1 + (int)(uniform() * 40);
    mlcp::dw_acc acc = mlcp::acc_zero(), sacc = mlcp::acc_zero();
    long double want = 0.0L, mag = 0.0L, swant = 0.0L, smag = 0.0L;
    for (int q = 0; q < nt; ++q) {
      const dw x = random_dw(10, false), y = random_dw(10, false);
      mlcp::acc_fma(acc, x, y);
      want += ld(x) * ld(y);
      mag += fabsl(ld(x) * ld(y));
      mlcp::acc_add(sacc, x);
      swant += ld(x);
      smag += fabsl(ld(x));
    }
    e_dot = std::fmax(e_dot, scaled(ld(mlcp::acc_value(acc)), want, mag));
    e_sum = std::fmax(e_sum, scaled(ld(mlcp::acc_value(sacc)), swant, smag));
  }
  report("acc_dot", e_dot);
  report("acc_sum", e_sum);
  report("add_f", e_addf);
  report("mul_f", e_mulf);
  report("from_double", e_conv);
  return 0;
}
