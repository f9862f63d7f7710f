// Correctly rounded log, sin/cos and acos for the trajectory.
//
// The reference computes its gas clocks (-tc log(1 - u)), Marsaglia normals
// (sqrt(-2 log s / s)) and cosine-law reflections (acos(sqrt u), cos and sin
// of the angles) with the host C library, whose results are the correctly
// rounded ones for all but ~0.1% of arguments.  CUDA's own functions are
// within an ulp but differ from them on ~0.3% (log) to ~20% (cos, sin, acos)
// of these arguments, and a trajectory grazing the ceiling turns such an ulp
// into a wall-time difference that can swap a gas collision and a wall hit,
// after which the particle consumes its random stream differently.  These
// functions evaluate the value in double-double arithmetic (~2^-85
// relative) and round it once, so they return the correctly rounded double
// except where the exact value lies within ~2^-85 of a rounding boundary.
//
// Methods (standard, from the mathematics):
//   log: x = 2^e m, m in [0.75, 1.5); m = (1 + t) / R with R from a 96-entry
//        table (R = 1 near m = 1), so log x = e ln 2 - log R + log1p(t),
//        |t| <= 2^-7, log1p by its Taylor series (terms to t^3 in
//        double-double, the rest to t^13 in double).
//   sin/cos: Cody-Waite reduction by pi/2 and by pi/64 with three-part
//        constants (exact products for the arguments used here, |x| < 2^20),
//        table of sin, cos(j pi / 64) in double-double, Taylor series of the
//        remainder (|s| <= pi/128) to s^11, angle addition in double-double.
//   acos: CUDA's acos as the start, one Newton step on cos(y) - x evaluated
//        with the double-double cos and sin, one rounding.
#pragma once

#include "st_crmath_tables.h"

namespace st {
namespace crm {

struct DD {
  double hi, lo;
};

// a + b exactly (Knuth), |a| and |b| in any order
__device__ __forceinline__ DD two_sum(double a, double b) {
  const double s = __dadd_rn(a, b);
  const double bb = __dsub_rn(s, a);
  const double e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, bb)), __dsub_rn(b, bb));
  return {s, e};
}
// a + b exactly when |a| >= |b| (Dekker)
__device__ __forceinline__ DD fast_two_sum(double a, double b) {
  const double s = __dadd_rn(a, b);
  return {s, __dsub_rn(b, __dsub_rn(s, a))};
}
// a * b exactly (the rounding error from one fused multiply-add)
__device__ __forceinline__ DD two_prod(double a, double b) {
  const double p = __dmul_rn(a, b);
  return {p, __fma_rn(a, b, -p)};
}
__device__ __forceinline__ DD dd_add(DD a, DD b) {
  DD s = two_sum(a.hi, b.hi);
  const DD t = two_sum(a.lo, b.lo);
  s = fast_two_sum(s.hi, __dadd_rn(s.lo, t.hi));
  return fast_two_sum(s.hi, __dadd_rn(s.lo, t.lo));
}
__device__ __forceinline__ DD dd_add_d(DD a, double b) {
  const DD s = two_sum(a.hi, b);
  return fast_two_sum(s.hi, __dadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ DD dd_mul(DD a, DD b) {
  const DD p = two_prod(a.hi, b.hi);
  return fast_two_sum(p.hi, __fma_rn(a.hi, b.lo, __fma_rn(a.lo, b.hi, p.lo)));
}
__device__ __forceinline__ DD dd_mul_d(DD a, double b) {
  const DD p = two_prod(a.hi, b);
  return fast_two_sum(p.hi, __fma_rn(a.lo, b, p.lo));
}
__device__ __forceinline__ DD dd_neg(DD a) { return {-a.hi, -a.lo}; }

// ---------------------------------------------------------------- log
// The three entry points are called, not inlined: they are rare next to the
// spin steps, and one copy of each keeps the trajectory code small.

// Natural logarithm of a positive normal double, correctly rounded (see the
// file comment); log(1) = 0.
static __device__ __noinline__ double cr_log(double x) {
  const long long bits = __double_as_longlong(x);
  int e = (int)((bits >> 52) & 0x7ff) - 1023;
  double m = __longlong_as_double((bits & 0x000fffffffffffffll) | 0x3ff0000000000000ll);  // [1, 2)
  if (m >= 1.5) {
    m = __dmul_rn(m, 0.5);
    e += 1;
  }
  const int j = (int)__dmul_rn(__dsub_rn(m, 0.75), 128.0);  // exact, 0..95
  const double r = kLogR[j];
  const DD p = two_prod(m, r);
  const DD t = two_sum(__dsub_rn(p.hi, 1.0), p.lo);  // m r - 1, exactly
  // log1p(t) = t - t^2/2 + t^3/3 - t^4/4 + ... + t^13/13
  const double z = t.hi;
  double tail = 1.0 / 13.0;
  tail = __fma_rn(tail, z, -1.0 / 12.0);
  tail = __fma_rn(tail, z, 1.0 / 11.0);
  tail = __fma_rn(tail, z, -1.0 / 10.0);
  tail = __fma_rn(tail, z, 1.0 / 9.0);
  tail = __fma_rn(tail, z, -1.0 / 8.0);
  tail = __fma_rn(tail, z, 1.0 / 7.0);
  tail = __fma_rn(tail, z, -1.0 / 6.0);
  tail = __fma_rn(tail, z, 1.0 / 5.0);
  tail = __fma_rn(tail, z, -1.0 / 4.0);
  const double z2 = __dmul_rn(z, z);
  tail = __dmul_rn(tail, __dmul_rn(z2, z2));
  const DD t2 = dd_mul(t, t);
  const DD t3 = dd_mul(t2, t);
  DD l = dd_add(t, {-0.5 * t2.hi, -0.5 * t2.lo});
  l = dd_add(l, dd_mul(t3, {kThirdHi, kThirdLo}));
  l = dd_add_d(l, tail);
  // + e ln 2 - log R
  const DD el = dd_add(two_prod((double)e, kLn2Hi), two_prod((double)e, kLn2Lo));
  const DD lr = {kLogL[j][0], kLogL[j][1]};
  const DD s = dd_add(dd_add(el, lr), l);
  return __dadd_rn(s.hi, s.lo);
}

// ---------------------------------------------------------------- sin, cos
// sin and cos of x, 0 <= |x| < 2^20, as double-double values.
__device__ __forceinline__ void sincos_dd(double x, DD& sn, DD& cs) {
  // x = k pi/2 + r
  const double k = rint(__dmul_rn(x, kTwoOverPi));
  const double r1 = __fma_rn(-k, kPio21, x);  // exact: k * kPio21 is exact and cancels
  DD r = two_sum(r1, __dmul_rn(-k, kPio22));  // k * kPio22 is exact
  r = dd_add(r, dd_neg(two_prod(k, kPio23)));
  // r = j pi/64 + s
  const double jd = rint(__dmul_rn(r.hi, kSixtyFourOverPi));
  DD s = dd_add(r, {__dmul_rn(-jd, kPio641), 0.0});
  s = dd_add(s, {__dmul_rn(-jd, kPio642), 0.0});
  s = dd_add(s, dd_neg(two_prod(jd, kPio643)));
  // sin s, cos s: Taylor series, |s| <= pi/128
  const DD s2 = dd_mul(s, s);
  const DD s3 = dd_mul(s2, s);
  const double w = s2.hi;
  double ps = -1.0 / 39916800.0;
  ps = __fma_rn(ps, w, 1.0 / 362880.0);
  ps = __fma_rn(ps, w, -1.0 / 5040.0);
  ps = __fma_rn(ps, w, 1.0 / 120.0);
  const double ts = __dmul_rn(ps, __dmul_rn(s3.hi, w));  // s^5 (1/120 - s^2/5040 + ...)
  DD ss = dd_add(s, dd_neg(dd_mul(s3, {kSixthHi, kSixthLo})));
  ss = dd_add_d(ss, ts);
  double pc = 1.0 / 40320.0;
  pc = __fma_rn(pc, w, -1.0 / 720.0);
  pc = __fma_rn(pc, w, 1.0 / 24.0);
  const double tc = __dmul_rn(pc, __dmul_rn(w, w));  // s^4 (1/24 - s^2/720 + s^4/40320)
  DD cc = dd_add({1.0, 0.0}, {-0.5 * s2.hi, -0.5 * s2.lo});
  cc = dd_add_d(cc, tc);
  // angle addition with the table at a = |j| pi / 64
  const int ja = (int)fabs(jd);
  DD sa = {kSinA[ja][0], kSinA[ja][1]};
  const DD ca = {kCosA[ja][0], kCosA[ja][1]};
  if (jd < 0.0) sa = dd_neg(sa);
  const DD sr = dd_add(dd_mul(sa, cc), dd_mul(ca, ss));
  const DD cr = dd_add(dd_mul(ca, cc), dd_neg(dd_mul(sa, ss)));
  // quadrant
  const int q = ((int)k) & 3;
  if (q == 0) {
    sn = sr; cs = cr;
  } else if (q == 1) {
    sn = cr; cs = dd_neg(sr);
  } else if (q == 2) {
    sn = dd_neg(sr); cs = dd_neg(cr);
  } else {
    sn = dd_neg(cr); cs = sr;
  }
}

// sin and cos of x, 0 <= |x| < 2^20, each correctly rounded (see the file comment).
static __device__ __noinline__ void cr_sincos(double x, double& s, double& c) {
  DD sn, cs;
  sincos_dd(x, sn, cs);
  s = __dadd_rn(sn.hi, sn.lo);
  c = __dadd_rn(cs.hi, cs.lo);
}

// ---------------------------------------------------------------- acos
// acos of x in [0, 1], correctly rounded (see the file comment).
static __device__ __noinline__ double cr_acos(double x) {
  if (x >= 1.0) return acos(x);  // 0 at 1, NaN above
  const double y0 = acos(x);
  DD sn, cs;
  sincos_dd(y0, sn, cs);
  const DD num = dd_add_d(cs, -x);  // cos(y0) - x
  const double d = __ddiv_rn(__dadd_rn(num.hi, num.lo), __dadd_rn(sn.hi, sn.lo));
  return __dadd_rn(y0, d);
}

}  // namespace crm
}  // namespace st
