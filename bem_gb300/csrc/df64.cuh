// Double-float ("df") arithmetic: a value is hi + lo with two FP32 numbers,
// |lo| <= ulp(hi) / 2, about 48 significant bits.  GB300 runs FP32 at 64x its
// FP64 rate, so FP64-class quadrature is cheaper in df on the FP32 pipes.
//
// Building blocks (published methods):
//   * TwoSum (Knuth), Fast2Sum (Dekker), TwoProduct via FMA - error-free
//     transformations;
//   * the "sloppy" df addition of Dekker / Bailey's double-double libraries
//     (error ~2^-47 of |a| + |b|) and the FMA-based df product;
//   * square root and reciprocal by one Newton step from the FP32 value
//     (Karp-Markstein form);
//   * sin, cos on [-pi/4, pi/4] and exp on [-ln2/2, ln2/2] by their Taylor
//     series (argument reduction by Cody-Waite in FP64 by the caller), the
//     high-order terms in FP32 where they are below 2^-25 of the result.
#pragma once

#include <cuda_runtime.h>

#include "df_constants.h"

namespace {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_make(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_to_double(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b| or a == 0
  const float s = a + b;
  return {s, b - (s - a)};
}

__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_mul_f(df a, float b) {
  const float p = a.hi * b;
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ df df_sqr(df a) {
  const float p = a.hi * a.hi;
  float e = fmaf(a.hi, a.hi, -p);
  e = fmaf(2.f * a.hi, a.lo, e);
  return fast_two_sum(p, e);
}
// a * 2^k for a float power of two p2 (exact)
__device__ __forceinline__ df df_scale2(df a, float p2) { return {a.hi * p2, a.lo * p2}; }

// sqrt(a), a > 0: s = a.hi * r (r ~ 1/sqrt(a.hi)), then s + (a - s^2) r / 2.
__device__ __forceinline__ df df_sqrt(df a) {
  const float r = rsqrtf(a.hi);
  const float s = a.hi * r;
  const df s2 = df_sqr({s, 0.f});
  const df d = df_sub(a, s2);  // small: a - s^2
  return fast_two_sum(s, 0.5f * d.hi * r);
}
// 1 / a: r = 1/a.hi, then r + r (1 - a r).
__device__ __forceinline__ df df_rcp(df a) {
  const float r = __frcp_rn(a.hi);
  const df ar = df_mul_f(a, r);
  const df e = df_add_f(df_neg(ar), 1.f);  // 1 - a r, small
  return fast_two_sum(r, r * e.hi);
}

// Taylor coefficient 1/n! as df (exact values from df_constants.h).
__device__ __forceinline__ df inv_fact(int n) { return {DF_FACT_HI[n], DF_FACT_LO[n]}; }

// sin r, cos r for |r| <= pi/4 + a little (df): Taylor series in s = r^2,
// sin up to r^17, cos up to r^18; terms below 2^-25 of the result in FP32.
__device__ __forceinline__ void df_sincos_reduced(df r, df &sn, df &cs) {
  const df s = df_sqr(r);
  const float sf = s.hi;
  // FP32 tails: sin coefficients of r^17 .. r^11, cos of r^18 .. r^12 (signs alternate)
  float ts = -inv_fact(17).hi;
  ts = fmaf(ts, sf, inv_fact(15).hi);
  ts = fmaf(ts, sf, -inv_fact(13).hi);
  ts = fmaf(ts, sf, inv_fact(11).hi);
  float tc = inv_fact(18).hi;
  tc = fmaf(tc, sf, -inv_fact(16).hi);
  tc = fmaf(tc, sf, inv_fact(14).hi);
  tc = fmaf(tc, sf, -inv_fact(12).hi);
  // df Horner for the leading terms
  df ps = {ts, 0.f};
  ps = df_add(df_mul(ps, s), df_neg(inv_fact(9)));
  ps = df_add(df_mul(ps, s), inv_fact(7));
  ps = df_add(df_mul(ps, s), df_neg(inv_fact(5)));
  ps = df_add(df_mul(ps, s), inv_fact(3));
  // sin = r - r s (1/3! - s (1/5! - ...)) : ps now holds -(coefficient series of r^3 term)/...
  // ps = -1/3! + s/5! - ... is the series of (sin r - r)/(r^3) with the sign folded:
  ps = df_neg(ps);
  sn = df_add(r, df_mul(df_mul(ps, s), r));
  df pc = {tc, 0.f};
  pc = df_add(df_mul(pc, s), inv_fact(10));
  pc = df_add(df_mul(pc, s), df_neg(inv_fact(8)));
  pc = df_add(df_mul(pc, s), inv_fact(6));
  pc = df_add(df_mul(pc, s), df_neg(inv_fact(4)));
  pc = df_add(df_mul(pc, s), inv_fact(2));
  // cos = 1 - s (1/2! - s/4! + ...)
  cs = df_add_f(df_neg(df_mul(pc, s)), 1.f);
}

// e^r - 1 for |r| <= 0.35 (df): Taylor series up to r^13, tail in FP32.
__device__ __forceinline__ df df_expm1_reduced(df r) {
  const float rf = r.hi;
  float t = inv_fact(13).hi;
  t = fmaf(t, rf, inv_fact(12).hi);
  t = fmaf(t, rf, inv_fact(11).hi);
  t = fmaf(t, rf, inv_fact(10).hi);
  t = fmaf(t, rf, inv_fact(9).hi);
  t = fmaf(t, rf, inv_fact(8).hi);
  df p = {t, 0.f};
  p = df_add(df_mul(p, r), inv_fact(7));
  p = df_add(df_mul(p, r), inv_fact(6));
  p = df_add(df_mul(p, r), inv_fact(5));
  p = df_add(df_mul(p, r), inv_fact(4));
  p = df_add(df_mul(p, r), inv_fact(3));
  p = df_add(df_mul(p, r), inv_fact(2));
  p = df_add_f(df_mul(p, r), 1.f);
  return df_mul(p, r);  // r (1 + r/2 + r^2/6 + ...)
}

// (cos x, sin x) for x given in FP64 (|x| < 2^20): quadrant reduction in FP64,
// the series in df.
__device__ __forceinline__ void df_sincos(double x, df &sn, df &cs) {
  const double n = rint(x * DF_TWO_OVER_PI);
  const double r = fma(-n, DF_PIO2_LO, fma(-n, DF_PIO2_HI, x));
  df s, c;
  df_sincos_reduced(df_make(r), s, c);
  const int q = ((int)n) & 3;
  if (q == 0) { sn = s; cs = c; }
  else if (q == 1) { sn = c; cs = df_neg(s); }
  else if (q == 2) { sn = df_neg(s); cs = df_neg(c); }
  else { sn = df_neg(c); cs = s; }
}

// e^x for x given in FP64 (-80 < x < 80): x = n ln2 + r in FP64, e^r in df.
__device__ __forceinline__ df df_exp(double x) {
  const double n = rint(x * DF_LOG2E);
  const double r = fma(-n, DF_LN2_LO, fma(-n, DF_LN2_HI, x));
  const df em1 = df_expm1_reduced(df_make(r));
  const df e = df_add_f(em1, 1.f);
  const float p2 = __int_as_float((127 + (int)n) << 23);
  return df_scale2(e, p2);
}

// x - n (c0 + c1 + c2 + c3) for an integer n, |n| < 2^8, with FP32 parts c0..c2
// of 16 bits (exact products) and a 24-bit c3.  When x.hi - n c0 cancels
// (Sterbenz) the first step is exact, so the reduced argument keeps ~2^-48 of
// its own size.
__device__ __forceinline__ df df_reduce(df x, float n, float c0, float c1, float c2, float c3) {
  df r = df_add_f(x, -n * c0);
  r = df_add_f(r, -n * c1);
  r = df_add_f(r, -n * c2);
  r.lo = fmaf(-n, c3, r.lo);
  return fast_two_sum(r.hi, r.lo);
}

// (sin x, cos x) for a df argument, |x| < 200 (quadrant count below 2^8),
// everything on the FP32 pipes.
__device__ __forceinline__ void df_sincos_df(df x, df &sn, df &cs) {
  const float n = rintf(x.hi * DF_TWO_OVER_PI_F);
  const df r = df_reduce(x, n, DF_PIO2_F0, DF_PIO2_F1, DF_PIO2_F2, DF_PIO2_F3);
  df s, c;
  df_sincos_reduced(r, s, c);
  const int q = ((int)n) & 3;
  if (q == 0) { sn = s; cs = c; }
  else if (q == 1) { sn = c; cs = df_neg(s); }
  else if (q == 2) { sn = df_neg(s); cs = df_neg(c); }
  else { sn = df_neg(c); cs = s; }
}

// e^x for a df argument, -85 < x < 85, on the FP32 pipes.
__device__ __forceinline__ df df_exp_df(df x) {
  const float n = rintf(x.hi * DF_LOG2E_F);
  const df r = df_reduce(x, n, DF_LN2_F0, DF_LN2_F1, DF_LN2_F2, DF_LN2_F3);
  const df e = df_add_f(df_expm1_reduced(r), 1.f);
  return df_scale2(e, __int_as_float((127 + (int)n) << 23));
}

__device__ __forceinline__ df df_abs(df a) { return a.hi < 0.f ? df_neg(a) : a; }

// log x, x > 0 with e^-85 < x < e^85: y0 = logf(x) (FP32), then one Newton
// step on e^y = x: t = x e^-y0 - 1 (small), log x = y0 + log(1 + t) with
// log(1 + t) = t - t^2/2 (the t^3 term is below 2^-48 for |t| < 2^-20).
__device__ __forceinline__ df df_log(df x) {
  const float y0 = logf(x.hi);
  const df e = df_exp_df({-y0, 0.f});
  const df t = df_add_f(df_mul(x, e), -1.f);
  const df u = df_add_f(t, -0.5f * t.hi * t.hi);
  return df_add_f(u, y0);
}

// atan2(y, x), (x, y) != (0, 0): t0 = atan2f(y, x) (FP32), then the exact
// correction t = t0 + atan(r), r = (y cos t0 - x sin t0) / (x cos t0 + y sin t0),
// with atan(r) = r for |r| < 2^-20 (the r^3 / 3 term is below 2^-60).
__device__ __forceinline__ df df_atan2(df y, df x) {
  const float t0 = atan2f(y.hi, x.hi);
  df s, c;
  df_sincos_df({t0, 0.f}, s, c);
  const df num = df_sub(df_mul(y, c), df_mul(x, s));
  const df den = df_add(df_mul(x, c), df_mul(y, s));
  if (den.hi == 0.f) return {t0, 0.f};
  return df_add_f(df_mul(num, df_rcp(den)), t0);
}

}  // namespace
