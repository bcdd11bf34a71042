// Host check of qvm_gb300/csrc/cplx.h's integer double -> double-float split
// against the FP64 form it replaces: hi = x truncated to 24 bits, lo =
// RN(x - hi) computed in FP64.  Built and run by test_dfloat_split.py.
#include <cmath>
#include <cstdio>
#include <random>

#include "cplx.h"

int main() {
  std::mt19937_64 g(1);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::uniform_int_distribution<int> E(-74, 127);
  long n = 0, bad = 0, outside = 0;
  for (long it = 0; it < 4000000; ++it) {
    double x = U(g) * std::ldexp(1.0, E(g));
    if (it % 5 == 0) x = std::ldexp(1.0, E(g)) * (U(g) < 0 ? -1 : 1);  // powers of two: r = 0
    if (it % 11 == 0) x = std::nextafter(x, 0.0);                        // all low bits set
    float hi, lo;
    if (!qvmg::df_split_int(x, hi, lo)) {
      ++outside;
      continue;
    }
    ++n;
    const float want_lo = (float)(x - (double)hi);
    const double back = (double)hi + (double)lo;
    if (qvmg::df_fbits(lo) != qvmg::df_fbits(want_lo) || std::fabs(back - x) > std::ldexp(std::fabs(x), -47))
      if (++bad < 5) std::printf("mismatch %a: hi %a lo %a want %a\n", x, hi, lo, want_lo);
  }
  // outside the range the caller falls back to the FP64 form
  float h, l;
  const bool tiny = qvmg::df_split_int(std::ldexp(1.0, -75), h, l);
  const bool zero = qvmg::df_split_int(0.0, h, l);
  const bool huge = qvmg::df_split_int(std::ldexp(1.0, 128), h, l);
  std::printf("checked %ld outside %ld mismatches %ld\n", n, outside, bad);
  return (bad || tiny || zero || huge || n < 3000000) ? 1 : 0;
}
