// dword.cuh -- double-word arithmetic: a value is an unevaluated sum hi + lo of two FP32 numbers
// with |lo| <= ulp(hi)/2, giving a ~48-bit significand computed entirely on the FP32 pipes.
//
// GB300's FP64 pipe runs at 1/69 of its FP32 rate (measured 503 GFMA/s vs 34.9 TFMA/s) and its
// FP64<->FP32 conversions run at the FP64 rate, so FP64-class accuracy is cheaper in double-word
// form. The building blocks are the published error-free transformations and double-word
// algorithms:
//   2Sum (Knuth, TAOCP vol. 2), Fast2Sum (Dekker 1971), Fast2Mult with FMA,
//   AccurateDWPlusDW (Alg. 6), SloppyDWPlusDW (Alg. 5), DWPlusFP (Alg. 4), DWTimesFP3 (Alg. 9)
//   and DWTimesDW3 (Alg. 12) of M. Joldes, J.-M. Muller, V. Popescu, "Tight and rigorous error
//   bounds for basic building blocks of double-word arithmetic", ACM TOMS 44(2), 2017 -- relative
//   errors <= 3u^2, (3u^2 of the operands' magnitudes), 2u^2, 2u^2, 4u^2 with u = 2^-24;
//   a fused multiply-add x*y + z built from the same transformations (6u^2 of |x y| + |z|) and a
//   two-term dot product x*y + z*w (6u^2 of |x y| + |z w|);
//   the reciprocal is one Newton-Raphson step r = t + t(1 - y t) from the FP32 reciprocal t.
// Values below ~2^-100 lose low-part bits to FP32 underflow; the solver only needs them to
// absolute accuracy.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

namespace sg {

struct dw {
  float hi, lo;
};

#define SG_HD __host__ __device__ __forceinline__

// Every operation below is rounded on its own, as the error-free transformations require: in
// device code through the _rn intrinsics, which the compiler never fuses into multiply-adds
// (nvcc fuses a plain a*b + c by default); in host code through plain operators, built with
// -ffp-contract=off.
#ifdef __CUDA_ARCH__
#define DW_ADD(a, b) __fadd_rn((a), (b))
#define DW_SUB(a, b) __fsub_rn((a), (b))
#define DW_MUL(a, b) __fmul_rn((a), (b))
#define DW_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#else
#define DW_ADD(a, b) ((a) + (b))
#define DW_SUB(a, b) ((a) - (b))
#define DW_MUL(a, b) ((a) * (b))
#define DW_FMA(a, b, c) fmaf((a), (b), (c))
#endif

SG_HD dw dw_make(float h, float l) { return dw{h, l}; }

// Fast2Sum: exact s + t = a + b when |a| >= |b| (or a's exponent is at least b's)
SG_HD dw fast2sum(float a, float b) {
  const float s = DW_ADD(a, b);
  const float z = DW_SUB(s, a);
  return dw{s, DW_SUB(b, z)};
}

// 2Sum: exact s + t = a + b for any a, b
SG_HD dw two_sum(float a, float b) {
  const float s = DW_ADD(a, b);
  const float ap = DW_SUB(s, b);
  const float bp = DW_SUB(s, ap);
  const float da = DW_SUB(a, ap);
  const float db = DW_SUB(b, bp);
  return dw{s, DW_ADD(da, db)};
}

// Fast2Mult: exact p + e = a * b (FMA)
SG_HD dw two_prod(float a, float b) {
  const float p = DW_MUL(a, b);
  return dw{p, DW_FMA(a, b, -p)};
}

// AccurateDWPlusDW
SG_HD dw dw_add(dw x, dw y) {
  const dw s = two_sum(x.hi, y.hi);
  const dw t = two_sum(x.lo, y.lo);
  const float c = DW_ADD(s.lo, t.hi);
  const dw v = fast2sum(s.hi, c);
  const float w = DW_ADD(t.lo, v.lo);
  return fast2sum(v.hi, w);
}

// SloppyDWPlusDW (Alg. 5 of Joldes, Muller, Popescu 2017): fewer operations. Its error is
// within ~3u^2 (|x| + |y|) for any signs, and so within ~3u^2 of the result when x and y have the
// same sign (no cancellation).
SG_HD dw dw_add_same(dw x, dw y) {
  const dw s = two_sum(x.hi, y.hi);
  const float v = DW_ADD(x.lo, y.lo);
  const float w = DW_ADD(s.lo, v);
  return fast2sum(s.hi, w);
}

SG_HD dw dw_neg(dw x) { return dw{-x.hi, -x.lo}; }
SG_HD dw dw_sub(dw x, dw y) { return dw_add(x, dw_neg(y)); }

// x*y + z in one renormalisation: the exact product of the high parts (Fast2Mult), its low part
// and the cross terms folded by FMA, then 2Sum with z's high part. Error within 6u^2 (|x y| +
// |z|): enough wherever the accuracy needed is relative to the operands' magnitudes rather than
// to a result that cancels (x.lo*y.lo, below u^2 |x y|, is left out).
SG_HD dw dw_fma(dw x, dw y, dw z) {
  const dw p = two_prod(x.hi, y.hi);
  const float t = DW_FMA(x.hi, y.lo, DW_FMA(x.lo, y.hi, p.lo));
  const dw s = two_sum(p.hi, z.hi);
  const float w = DW_ADD(DW_ADD(t, z.lo), s.lo);
  return fast2sum(s.hi, w);
}

// dw_fma(x, y, 0) without the operations on the zero addend (the same value)
SG_HD dw dw_fma0(dw x, dw y) {
  const dw p = two_prod(x.hi, y.hi);
  return fast2sum(p.hi, DW_FMA(x.hi, y.lo, DW_FMA(x.lo, y.hi, p.lo)));
}

// x*y + z*w: both high-part products exact (Fast2Mult), their low parts and the cross terms
// folded by FMA, one 2Sum of the high parts and one renormalisation -- 19 FP32 operations
// against 24 for dw_fma(x, y, dw_mul(z, w)). Error within ~6u^2 (|x y| + |z w|) (the lo*lo terms,
// below u^2 of each product, are left out, as in dw_fma).
SG_HD dw dw_dot2(dw x, dw y, dw z, dw w) {
  const dw p = two_prod(x.hi, y.hi);
  const dw q = two_prod(z.hi, w.hi);
  const dw s = two_sum(p.hi, q.hi);
  const float t = DW_FMA(x.hi, y.lo, DW_FMA(x.lo, y.hi, p.lo));
  const float u = DW_FMA(z.hi, w.lo, DW_FMA(z.lo, w.hi, q.lo));
  return fast2sum(s.hi, DW_ADD(DW_ADD(t, u), s.lo));
}

// DWPlusFP
SG_HD dw dw_add_f(dw x, float y) {
  const dw s = two_sum(x.hi, y);
  const float v = DW_ADD(x.lo, s.lo);
  return fast2sum(s.hi, v);
}

// DWTimesFP3
SG_HD dw dw_mul_f(dw x, float y) {
  const dw c = two_prod(x.hi, y);
  const float cl3 = DW_FMA(x.lo, y, c.lo);
  return fast2sum(c.hi, cl3);
}

// DWTimesDW3
SG_HD dw dw_mul(dw x, dw y) {
  const dw c = two_prod(x.hi, y.hi);
  const float tl0 = DW_MUL(x.lo, y.lo);
  const float tl1 = DW_FMA(x.hi, y.lo, tl0);
  const float cl2 = DW_FMA(x.lo, y.hi, tl1);
  const float cl3 = DW_ADD(c.lo, cl2);
  return fast2sum(c.hi, cl3);
}

// 1/y: approximate FP32 reciprocal t (a few ulps), then r = t + t*(1 - y*t) with y*t formed in
// double-word; the Newton step squares the relative error of t.
SG_HD dw dw_rcp(dw y) {
#ifdef __CUDA_ARCH__
  const float t = __fdividef(1.0f, y.hi);
#else
  const float t = 1.0f / y.hi;
#endif
  const dw p = dw_mul_f(y, t);               // y*t ~ 1
  const float e = DW_SUB(DW_SUB(1.0f, p.hi), p.lo);  // 1 - p.hi is exact (Sterbenz)
  return fast2sum(t, DW_MUL(t, e));
}

SG_HD dw dw_div(dw x, dw y) { return dw_mul(x, dw_rcp(y)); }

SG_HD dw dw_abs(dw x) { return x.hi < 0.0f || (x.hi == 0.0f && x.lo < 0.0f) ? dw_neg(x) : x; }
SG_HD dw dw_max0(dw x) { return x.hi > 0.0f ? x : dw{0.0f, 0.0f}; }
SG_HD bool dw_gt0(dw x) { return x.hi > 0.0f; }

// conversions (FP64 pipe: only at set-up and at the API boundary)
SG_HD dw dw_from_double(double v) {
  const float h = (float)v;
  return dw{h, (float)(v - (double)h)};
}
SG_HD double dw_to_double(dw x) { return (double)x.hi + (double)x.lo; }

// The same conversions for the layout transforms at the API boundary, which convert every cell
// once per call: there the FP64 pipe (which also carries the FP64<->FP32 conversions, 3-4 per
// value above) set the time. These do the rounding with integer operations on the bits and give
// the bits of dw_from_double / dw_to_double for every input; exponents outside the range handled
// here (zeros, subnormal results, overflow, infinities, NaNs) take the conversions above.
SG_HD unsigned long long dw_dbits(double v) {
#ifdef __CUDA_ARCH__
  return (unsigned long long)__double_as_longlong(v);
#else
  unsigned long long u;
  memcpy(&u, &v, 8);
  return u;
#endif
}
SG_HD double dw_bitsd(unsigned long long u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double v;
  memcpy(&v, &u, 8);
  return v;
#endif
}
SG_HD unsigned int dw_fbits(float v) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(v);
#else
  unsigned int u;
  memcpy(&u, &v, 4);
  return u;
#endif
}
SG_HD float dw_bitsf(unsigned int u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float v;
  memcpy(&v, &u, 4);
  return v;
#endif
}

// v = (-1)^s 2^E 1.m with E in [-97, 126]: hi = RN(v) rounds the 53-bit significand to 24 bits
// (to nearest, ties to even; a carry out of the top bit raises the exponent); v - hi is exactly
// r 2^(E-52) with the remainder |r| <= 2^28, and lo = RN(r) * 2^(E-52), the one rounding of the
// exact value: an int-to-float conversion of r (exact below 2^24), then a product by a power of
// two that is exact whenever it is normal, which |r| >= 2^24 and E >= -97 ensure.
SG_HD dw dw_from_double_int(double v) {
  const unsigned long long u = dw_dbits(v);
  const int e = (int)((u >> 52) & 0x7FF);
  if (e < 1023 - 97 || e > 1023 + 126) return dw_from_double(v);
  const unsigned long long full = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  unsigned int keep = (unsigned int)(full >> 29);
  const int rem = (int)(full & 0x1FFFFFFFull);
  const bool up = rem > 0x10000000 || (rem == 0x10000000 && (keep & 1u));
  keep += up ? 1u : 0u;
  unsigned int ef = (unsigned int)(e - 1023 + 127);
  if (keep >> 24) {
    keep >>= 1;
    ++ef;
  }
  const unsigned int sgn = (unsigned int)(u >> 63);
  const float hi = dw_bitsf((sgn << 31) | (ef << 23) | (keep & 0x7FFFFFu));
  int r = up ? rem - 0x20000000 : rem;
  if (sgn) r = -r;
  const int k = e - 1023 - 52;  // in [-149, 74]
  const float scale = k >= -126 ? dw_bitsf((unsigned int)(k + 127) << 23) : dw_bitsf(1u << (k + 149));
#ifdef __CUDA_ARCH__
  const float rf = __int2float_rn(r);
#else
  const float rf = (float)r;
#endif
  return dw{hi, DW_MUL(rf, scale)};
}

// float -> double by moving the fields (normal numbers and zeros; others by conversion)
SG_HD double dw_f2d_int(float f) {
  const unsigned int u = dw_fbits(f);
  const unsigned int e = (u >> 23) & 0xFFu;
  const unsigned long long s = (unsigned long long)(u >> 31) << 63;
  if ((u & 0x7FFFFFFFu) == 0u) return dw_bitsd(s);
  if (e == 0u || e == 0xFFu) return (double)f;
  return dw_bitsd(s | ((unsigned long long)(e - 127u + 1023u) << 52) | ((unsigned long long)(u & 0x7FFFFFu) << 29));
}
SG_HD double dw_to_double_int(dw x) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(dw_f2d_int(x.hi), dw_f2d_int(x.lo));
#else
  return dw_f2d_int(x.hi) + dw_f2d_int(x.lo);
#endif
}

#undef SG_HD
#undef DW_ADD
#undef DW_SUB
#undef DW_MUL
#undef DW_FMA

}  // namespace sg
