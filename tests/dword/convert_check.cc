// Host check of the integer-rounding conversions in csrc/dword.cuh: dw_from_double_int and
// dw_to_double_int must give the bits of dw_from_double and dw_to_double for every input.
// Prints the number of inputs checked and of mismatches (compiled and run by tests/test_dword.py).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "dword.cuh"

using sg::dw;

static unsigned long long bits(double v) { unsigned long long u; std::memcpy(&u, &v, 8); return u; }
static unsigned int fbits(float v) { unsigned int u; std::memcpy(&u, &v, 4); return u; }
static double dbl(unsigned long long u) { double v; std::memcpy(&v, &u, 8); return v; }

int main() {
  std::mt19937_64 g(2024);
  long long checked = 0, bad_from = 0, bad_to = 0;
  auto check_from = [&](double v) {
    const dw a = sg::dw_from_double(v), b = sg::dw_from_double_int(v);
    ++checked;
    if (fbits(a.hi) != fbits(b.hi) || fbits(a.lo) != fbits(b.lo)) {
      if (bad_from < 5) std::printf("from_double mismatch: %a -> (%a, %a) vs (%a, %a)\n", v, a.hi, a.lo, b.hi, b.lo);
      ++bad_from;
    }
  };
  auto check_to = [&](dw x) {
    const double a = sg::dw_to_double(x), b = sg::dw_to_double_int(x);
    ++checked;
    if (bits(a) != bits(b) && !(std::isnan(a) && std::isnan(b))) {
      if (bad_to < 5) std::printf("to_double mismatch: (%a, %a) -> %a vs %a\n", x.hi, x.lo, a, b);
      ++bad_to;
    }
  };
  // every binary exponent of the double range, random significands and signs
  for (int e = 0; e < 2047; ++e)
    for (int k = 0; k < 2000; ++k) {
      const unsigned long long u = ((g() & 1ull) << 63) | ((unsigned long long)e << 52) | (g() & 0xFFFFFFFFFFFFFull);
      const double v = dbl(u);
      check_from(v);
      check_to(sg::dw_from_double(v));
    }
  // ties and near-ties of the 24-bit rounding, both parities, with a carry out of the top bit
  for (int e = 1023 - 100; e <= 1023 + 127; ++e)
    for (int k = 0; k < 400; ++k) {
      unsigned long long m = g() & 0xFFFFFFFFFFFFFull;
      m = (m & ~0x1FFFFFFFull) | (k % 4 == 0 ? 0x10000000ull : k % 4 == 1 ? 0x0FFFFFFFull : k % 4 == 2 ? 0x10000001ull : 0ull);
      if (k % 16 == 5) m |= 0xFFFFFE0000000ull;  // all-ones top: rounding up carries into the exponent
      const double v = dbl(((g() & 1ull) << 63) | ((unsigned long long)e << 52) | m);
      check_from(v);
    }
  // special values
  const double sp[] = {0.0, -0.0, std::numeric_limits<double>::infinity(), -std::numeric_limits<double>::infinity(),
                       std::numeric_limits<double>::quiet_NaN(), std::numeric_limits<double>::denorm_min(),
                       std::numeric_limits<double>::min(), std::numeric_limits<double>::max(), 3.4028234663852886e38,
                       3.4028235677973366e38, 1.1754943508222875e-38, 1.401298464324817e-45, 7.0e-46, 1.0, -1.0};
  for (double v : sp) {
    check_from(v);
    check_to(sg::dw_from_double(v));
  }
  // arbitrary float pairs, including subnormals, zeros and unnormalised pairs
  for (int k = 0; k < 2000000; ++k) {
    const float a = sg::dw_bitsf((unsigned int)g()), b = sg::dw_bitsf((unsigned int)g());
    check_to(dw{a, b});
    check_to(dw{a, 0.0f});
  }
  std::printf("checked %lld from_double_mismatches %lld to_double_mismatches %lld\n", checked, bad_from, bad_to);
  return (bad_from || bad_to) ? 1 : 0;
}
