"""mlcp_gb300/csrc/fastdiv.cuh (division by a run-time invariant divisor as a
multiply-high and two shifts, the index splits of the Gram-Schmidt kernel):
the header itself, compiled on the host with g++, against the plain integer
division.  Exhaustive for divisors 1..4096 and numerators below 2^16, then
two million random 32-bit numerators with random divisors below 2^31 and the
edge numerators 0, 1, d - 1, d, d + 1, 2^31 - 1, 2^31 and 2^32 - 1.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHECK = r"""
#include <cstdio>
#include <random>
#include "fastdiv.cuh"
int main() {
  long long bad = 0, checks = 0;
  for (unsigned d = 1; d <= 4096; ++d) {
    mlcp::FastDiv f(d);
    for (unsigned n = 0; n < (1u << 16); ++n) {
      int q, r;
      f.divmod(n, &q, &r);
      if ((unsigned)q != n / d || (unsigned)r != n % d) ++bad;
      ++checks;
    }
  }
  std::mt19937_64 rng(1);
  for (int k = 0; k < 2000000; ++k) {
    unsigned d = (unsigned)(rng() % ((1u << 31) - 1)) + 1;
    if (k & 1) d = (unsigned)(rng() % 100000) + 1;
    mlcp::FastDiv f(d);
    const unsigned edges[] = {(unsigned)rng(), 0u, 1u, d - 1, d, d + 1, 0x7fffffffu, 0x80000000u, 0xffffffffu};
    for (unsigned n : edges) {
      if (f.div(n) != n / d) ++bad;
      ++checks;
    }
  }
  std::printf("%lld %lld\n", bad, checks);
  return 0;
}
"""


def test_fastdiv_matches_integer_division(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    src = tmp_path / "check.cpp"
    src.write_text(CHECK)
    exe = tmp_path / "check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "mlcp_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    bad, checks = int(out[0]), int(out[1])
    assert checks > 280_000_000
    assert bad == 0
