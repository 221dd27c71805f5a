// Host check of the double-word building blocks in csrc/dword.cuh against long-double references
// (compiled and run by tests/test_dword.py). For each operation it prints the worst error over
// random operands, in units of u^2 (u = 2^-24), measured against the bound the kernels rely on:
//   add, mul, rcp, div, add_same (same signs), add_f, mul_f: relative to the exact result
//   fma, dot2, add_same (any signs): relative to the operands' magnitudes (|x y| + |z|,
//   |x y| + |z w|, |x| + |y|)
#include <cmath>
#include <cstdio>
#include <random>

#include "dword.cuh"

using sg::dw;
typedef long double LD;

static LD val(dw x) { return (LD)x.hi + (LD)x.lo; }
static dw mk(std::mt19937_64& g, bool neg_ok) {
  std::uniform_real_distribution<double> m(0.5, 1.0);
  std::uniform_int_distribution<int> e(-30, 30);
  double v = std::ldexp(m(g), e(g));
  if (neg_ok && (g() & 1)) v = -v;
  return sg::dw_from_double(v);
}

int main() {
  std::mt19937_64 g(12345);
  const LD u2 = std::ldexp((LD)1, -48);
  double w[10] = {0};
  const char* names[10] = {"add", "add_same_same_sign", "add_same_any_sign_vs_magnitudes", "mul", "rcp", "div",
                           "fma_vs_magnitudes", "add_f", "mul_f", "dot2_vs_magnitudes"};
  for (int it = 0; it < 2000000; ++it) {
    dw x = mk(g, true), y = mk(g, true), z = mk(g, true);
    if (it % 4 == 0) {  // near-cancelling pairs
      y = sg::dw_neg(sg::dw_add_f(x, std::ldexp((float)((g() % 1000) + 1), -40) * x.hi));
    }
    LD ex;
    ex = val(x) + val(y);
    if (ex != 0) w[0] = std::fmax(w[0], (double)(fabsl(val(sg::dw_add(x, y)) - ex) / fabsl(ex) / u2));
    dw xa = sg::dw_abs(x), ya = sg::dw_abs(y);
    ex = val(xa) + val(ya);
    w[1] = std::fmax(w[1], (double)(fabsl(val(sg::dw_add_same(xa, ya)) - ex) / ex / u2));
    ex = val(x) + val(y);
    w[2] = std::fmax(w[2], (double)(fabsl(val(sg::dw_add_same(x, y)) - ex) / (fabsl(val(x)) + fabsl(val(y))) / u2));
    ex = val(x) * val(y);
    w[3] = std::fmax(w[3], (double)(fabsl(val(sg::dw_mul(x, y)) - ex) / fabsl(ex) / u2));
    ex = 1.0L / val(y);
    w[4] = std::fmax(w[4], (double)(fabsl(val(sg::dw_rcp(y)) - ex) / fabsl(ex) / u2));
    ex = val(x) / val(y);
    w[5] = std::fmax(w[5], (double)(fabsl(val(sg::dw_div(x, y)) - ex) / fabsl(ex) / u2));
    dw zz = (it % 4 == 1) ? sg::dw_neg(sg::dw_mul(x, y)) : z;  // cancelling addend too
    ex = val(x) * val(y) + val(zz);
    w[6] = std::fmax(w[6], (double)(fabsl(val(sg::dw_fma(x, y, zz)) - ex) / (fabsl(val(x) * val(y)) + fabsl(val(zz))) / u2));
    ex = val(x) + (LD)y.hi;
    if (ex != 0) w[7] = std::fmax(w[7], (double)(fabsl(val(sg::dw_add_f(x, y.hi)) - ex) / fabsl(ex) / u2));
    ex = val(x) * (LD)y.hi;
    w[8] = std::fmax(w[8], (double)(fabsl(val(sg::dw_mul_f(x, y.hi)) - ex) / fabsl(ex) / u2));
    // x*y + z*w, with near-cancelling second products in half of the draws
    dw zw = mk(g, true), ww = mk(g, true);
    if (it % 2 == 0) {
      zw = sg::dw_neg(x);
      ww = sg::dw_add_f(y, std::ldexp((float)((g() % 1000) + 1), -40) * y.hi);
    }
    ex = val(x) * val(y) + val(zw) * val(ww);
    w[9] = std::fmax(w[9], (double)(fabsl(val(sg::dw_dot2(x, y, zw, ww)) - ex) /
                                    (fabsl(val(x) * val(y)) + fabsl(val(zw) * val(ww))) / u2));
  }
  for (int k = 0; k < 10; ++k) std::printf("%s %.3f\n", names[k], w[k]);
  return 0;
}
