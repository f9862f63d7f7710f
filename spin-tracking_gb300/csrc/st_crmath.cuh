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
// functions evaluate the value in double-double arithmetic (~2^-67 relative
// or better) and round it once, so they return the correctly rounded double
// except where the exact value lies that close to a rounding boundary (about
// one argument in 10^4, against the host library's own ~10^-3).
//
// Methods (standard, from the mathematics):
//   log: x = 2^e m, m in [0.75, 1.5); m = (1 + t) / R with R from a 96-entry
//        table (R = 1 near m = 1), so log x = e ln 2 - log R + log1p(t),
//        |t| <= 2^-7, log1p by its Taylor series (terms to t^3 in
//        double-double, the rest to t^13 in double).
//   sin/cos: Cody-Waite reduction by pi/2 and by pi/256 with three-part
//        constants (exact products for the arguments used here, |x| < 2^20),
//        table of sin, cos(j pi / 256) in double-double, Taylor series of the
//        remainder (|s| <= pi/512) in double, angle addition with the leading
//        products exact (~2^-67 relative before the rounding).
//   acos: CUDA's acos as the start, one Newton step on cos(y) - x evaluated
//        with the double-double cos and sin, one rounding; the reflection's
//        sin and cos of the result reuse that evaluation when it rounds to
//        the start.
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
// sin and cos of x, 0 <= |x| < 2^20, as double-double values accurate to
// ~2^-67 relative.
__device__ __forceinline__ void sincos_dd(double x, DD& sn, DD& cs) {
  // x = k pi/2 + r, r as double-double (k * kPio21 and k * kPio22 are exact)
  const double k = rint(__dmul_rn(x, kTwoOverPi));
  const double r1 = __fma_rn(-k, kPio21, x);
  DD r = two_sum(r1, __dmul_rn(-k, kPio22));
  r = dd_add(r, dd_neg(two_prod(k, kPio23)));
  // r = j pi/256 + s, |s| <= pi/512 (j * kPio2561 and j * kPio2562 are exact)
  const double jd = rint(__dmul_rn(r.hi, k256OverPi));
  DD s = two_sum(__fma_rn(-jd, kPio2561, r.hi), __dmul_rn(-jd, kPio2562));
  s = dd_add_d(s, r.lo);
  const double sh = s.hi, sl = __fma_rn(-jd, kPio2563, s.lo);
  // sin s - s and cos s - 1 by their Taylor series in double (to s^7 and s^6)
  const double z = __dmul_rn(sh, sh);
  const double sp = __dmul_rn(__dmul_rn(sh, z), __fma_rn(z, __fma_rn(z, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0));
  const double cp = __fma_rn(-sh, sl, __dmul_rn(z, __fma_rn(z, __fma_rn(z, -1.0 / 720.0, 1.0 / 24.0), -0.5)));
  // angle addition with the table at a = j pi / 256: the leading products
  // exact, the small terms in double
  const int ja = (int)fabs(jd);
  double sah = kSinA[ja][0], sal = kSinA[ja][1];
  if (jd < 0.0) {
    sah = -sah;
    sal = -sal;
  }
  const double cah = kCosA[ja][0], cal = kCosA[ja][1];
  const double ss = __dadd_rn(sl, sp);  // sin s - sh
  // sin(a + s) = sin a + cos a sh + [cos a (sin s - sh) + sin a (cos s - 1)]
  const DD m = two_prod(cah, sh);
  const DD hs = two_sum(sah, m.hi);
  const double ts = __dadd_rn(__dadd_rn(m.lo, sal),
                              __fma_rn(cal, sh, __fma_rn(sah, cp, __dmul_rn(cah, ss))));
  const DD sr = fast_two_sum(hs.hi, __dadd_rn(hs.lo, ts));
  // cos(a + s) = cos a - sin a sh + [cos a (cos s - 1) - sin a (sin s - sh)]
  const DD m2 = two_prod(-sah, sh);
  const DD hc = two_sum(cah, m2.hi);
  const double tc = __dadd_rn(__dadd_rn(m2.lo, cal),
                              __fma_rn(-sal, sh, __fma_rn(cah, cp, __dmul_rn(-sah, ss))));
  const DD cr = fast_two_sum(hc.hi, __dadd_rn(hc.lo, tc));
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
// y = acos(x) for x in [0, 1], correctly rounded, with sin(y) and cos(y)
// correctly rounded too (a cosine-law reflection needs all three).  CUDA's
// acos gives y0; one Newton step on cos(y) - x with the double-double sin and
// cos of y0 gives y; when y rounds to y0 (most arguments) those sin and cos
// are y's, else they are evaluated again.
static __device__ __noinline__ void cr_acos_sincos(double x, double& y, double& sy, double& cy) {
  const double y0 = acos(x);
  DD sn, cs;
  sincos_dd(y0, sn, cs);
  if (x >= 1.0 || x != x) {  // acos(1) = 0 exactly; NaN passes through
    y = y0;
  } else {
    const double num = __dadd_rn(__dsub_rn(cs.hi, x), cs.lo);  // cos(y0) - x
    y = __dadd_rn(y0, __ddiv_rn(num, __dadd_rn(sn.hi, sn.lo)));
  }
  if (y != y0) sincos_dd(y, sn, cs);
  sy = __dadd_rn(sn.hi, sn.lo);
  cy = __dadd_rn(cs.hi, cs.lo);
}

static __device__ __noinline__ double cr_acos(double x) {
  double y, sy, cy;
  cr_acos_sincos(x, y, sy, cy);
  return y;
}

}  // namespace crm
}  // namespace st
