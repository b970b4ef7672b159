// FP64 reciprocal, square root, exp and log with fewer FP64-pipe operations than the
// correctly rounded library calls, for the FP64-pipe-bound column physics
// (GB300 issues FP64 at a small fraction of its FP32 rate).  Each result is
// within about 1.5 units in the last place of the exact value for normal
// inputs in the stated ranges; outside them the library call is taken (the
// range tests are integer compares on the exponent field, so they cost no
// FP64 operation).  Seeds and table indexes come from the integer pipe and
// the FP32 special-function unit; the FP64 work is:
//   rcp  3 DFMA: FP32 seed y0 (relative error e0 < 2^-21), then
//        y = y0 + y0 (e + e^2), e = 1 - x y0 (cubic Newton step, error
//        about e0^3 plus the final rounding);
//   sqrt 6 operations from an FP32 reciprocal-square-root seed (below);
//   exp  10 operations, the table-driven method of P. T. P. Tang, "Table-driven
//        implementation of the exponential function in IEEE floating-point
//        arithmetic", ACM TOMS 15 (1989): x = (64 m + j) ln2/64 + r,
//        |r| <= ln2/128, exp x = 2^m 2^(j/64) (1 + p(r)), p the Taylor
//        polynomial to r^5 (truncation below 4e-17), 2^m added to the
//        exponent field;
//   log  14 operations, the table-driven method of P. T. P. Tang, "Table-driven
//        implementation of the logarithm function in IEEE floating-point
//        arithmetic", ACM TOMS 16 (1990): x = 2^m Y, F = 1 + j/128 nearest
//        to Y, f = Y - F (exact), u = f / F (|u| <= 2^-8),
//        log x = m ln2 + ln F + log1p(u), log1p by its series to u^7
//        (truncation below 2^-67 absolute); m ln2 and ln F carry their
//        rounding remainders, so x just below 1 (m = -1, F near 2) keeps
//        full relative accuracy.
// Tables (fp64_tables.cuh, from gen_fp64_tables.py) are doubles nearest to
// the exact values, read through the read-only cache.
#pragma once

#include <cuda_runtime.h>

#include "fp64_tables.cuh"

namespace dccm {
namespace fp64 {

// FP32 image of x, mantissa truncated to 23 bits: valid while the exponent
// is in FP32's normal range.
__device__ __forceinline__ float f32_image(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned mag = __funnelshift_l(lo, (hi & 0x7FFFFFFFu) - 0x38000000u, 3);
  return __uint_as_float(mag | (hi & 0x80000000u));
}

// Exact widening of a normal FP32 value.
__device__ __forceinline__ double f64_of_normal(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned hi = (((b & 0x7FFFFFFFu) >> 3) + 0x38000000u) | (b & 0x80000000u);
  return __hiloint2double((int)hi, (int)(b << 29));
}

// 1 / x.  The seed path needs the FP32 image of x and of 1/x normal:
// biased FP64 exponent in [898, 1149] (|x| in [2^-125, 2^127)).
__device__ __forceinline__ double rcp(double x) {
  const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7FFu;
  if (e - 898u >= 252u) return 1.0 / x;
  float yf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(f32_image(x)));
  const double y = f64_of_normal(yf);
  const double err = fma(-x, y, 1.0);
  return fma(y, fma(err, err, err), y);
}

// a / b as a (1 / b): one more rounding than a division.
__device__ __forceinline__ double div(double a, double b) { return a * rcp(b); }

// a / b from rb = rcp(b) with Markstein's correction (P. Markstein, "Computation
// of elementary functions on the IBM RISC System/6000 processor", IBM J. Res.
// Dev. 34 (1990)): q = a rb, r = a - b q (exact with an FMA), q + r rb.  With
// rb within half an ulp of 1/b this is the correctly rounded quotient; 3
// FP64 operations when rb is shared by several divisions by b.
__device__ __forceinline__ double div_rb(double a, double b, double rb) {
  const double q = a * rb;
  return fma(fma(-b, q, a), rb, q);
}

// sqrt(x), and h within about 2 ulp of 1 / (2 sqrt x), by Goldschmidt's
// coupled iteration (R. E. Goldschmidt, "Applications of division by
// convergence", MIT thesis, 1964) from the FP32 seed y0 ~ 1/sqrt(x):
// s = x y0, h = y0 / 2, then twice r = 1/2 - s h, s += s r, h += h r
// (the second h update only when h is used).  6 FP64 operations for sqrt.
// Seed path: biased exponent in [898, 1149], positive x; otherwise the
// library sqrt.
__device__ __forceinline__ double sqrt_h(double x, double &h) {
  const unsigned e = (unsigned)__double2hiint(x) >> 20;  // the sign bit included
  if (e - 898u >= 252u) {
    const double s = ::sqrt(x);
    h = 0.5 / s;
    return s;
  }
  float y0;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y0) : "f"(f32_image(x)));
  double s = x * f64_of_normal(y0);
  double hh = f64_of_normal(0.5f * y0);
  double r = fma(-s, hh, 0.5);
  s = fma(s, r, s);
  hh = fma(hh, r, hh);
  r = fma(-s, hh, 0.5);
  h = fma(hh, r, hh);
  return fma(s, r, s);
}
__device__ __forceinline__ double sqrt(double x) {
  double h;
  return sqrt_h(x, h);
}

// e^x for |x| < 512 (biased exponent below 1032; the result stays normal).
__device__ __forceinline__ double exp(double x) {
  const unsigned e = ((unsigned)__double2hiint(x) >> 20) & 0x7FFu;
  if (e >= 1032u) return ::exp(x);
  constexpr double SHIFTER = 0x1.8p52;  // t's last place is 1: N = round(64 x / ln2) in its low word
  const double t = fma(x, INV_LN2_64, SHIFTER);
  const int N = __double2loint(t);
  const double Nd = t - SHIFTER;
  double r = fma(-Nd, LN2_64_HI, x);
  r = fma(-Nd, LN2_64_LO, r);
  double q = fma(r, 1.0 / 120.0, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  const double p = fma(r * r, q, r);
  const double S = __ldg(EXP2_64 + (N & 63));
  const double y = fma(S, p, S);
  return __hiloint2double(__double2hiint(y) + ((N >> 6) << 20), __double2loint(y));
}

// ln x for positive normal finite x.
__device__ __forceinline__ double log(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned e = hi >> 20;  // the sign bit included: negative x fails the test
  if (e - 1u >= 2046u) return ::log(x);
  const unsigned mant = hi & 0xFFFFFu;
  const unsigned j = (mant + (1u << 12)) >> 13;  // 0 .. 128
  const double Y = __hiloint2double((int)(0x3FF00000u | mant), (int)lo);
  const double F = __hiloint2double((int)(0x3FF00000u + (j << 13)), 0);
  const double f = Y - F;
  const double2 T = __ldg(LOG_F128 + j);
  const double u = f * T.x;
  double q = fma(u, 1.0 / 7.0, -1.0 / 6.0);
  q = fma(q, u, 1.0 / 5.0);
  q = fma(q, u, -0.25);
  q = fma(q, u, 1.0 / 3.0);
  q = fma(q, u, -0.5);
  const double p = fma(u * u, q, u);
  // m as a double without a conversion instruction: (2^52 + 2^31 + m) - (2^52 + 2^31)
  const double md = __hiloint2double(0x43300000, (int)(0x80000000u + (e - 1023u))) - 0x1.00000800p52;
  // m ln2 + ln F in a leading part (exact when the two nearly cancel, x
  // just below 1) and the rest, so that the cancellation loses nothing
  const double A = fma(md, LN2, T.y);
  const double B = fma(md, LN2_LO, __ldg(LOG_F128_LO + j)) + p;
  return A + B;
}

}  // namespace fp64
}  // namespace dccm
