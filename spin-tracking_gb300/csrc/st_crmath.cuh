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
// functions return the correctly rounded double (Ziv's strategy): a fast
// evaluation in double-double arithmetic with a stated error bound, a rounding
// test that accepts its result when no rounding boundary lies within that
// bound, and otherwise (a small fraction of a percent of arguments) an
// accurate evaluation to ~2^-100 relative, rounded once.  The accurate result
// is wrong only if the exact value lies within ~2^-96 of a midpoint between
// doubles (about one argument in 2^43).
//
// Methods (standard, from the mathematics):
//   log: x = 2^e m, m in [0.75, 1.5); m = (1 + t) / R with R from a 96-entry
//        table (R = 1 near m = 1), so log x = e ln 2 - log R + log1p(t),
//        |t| <= 2^-7, log1p by its Taylor series (fast: terms to t^3 in
//        double-double, the rest to t^13 in double; accurate: all terms to
//        t^15 in double-double).
//   sin/cos: Cody-Waite reduction by pi/2 and by pi/256 with three-part
//        constants (four-part in the accurate path; exact products for the
//        arguments used here, |x| < 2^20), table of sin, cos(j pi / 256) in
//        double-double, Taylor series of the remainder (|s| <= pi/512; fast:
//        in double, accurate: in double-double to s^15), angle addition.
//   acos: CUDA's acos as the start y0 and one Newton step on cos(y) = x, whose
//        residual is formed without cancellation: (1 - x) - 2 sin^2(y0 / 2)
//        for x >= 1/2 (1 - x is exact there), cos(y0) - x below; the accurate
//        path repeats the step twice in double-double.  The reflection's sin
//        and cos of the result reuse the step's evaluation when it rounds to
//        y0, each with its own rounding test.
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
__device__ __forceinline__ DD dd_mul_pow2(DD a, double p) { return {a.hi * p, a.lo * p}; }  // exact
// hi = RN(hi + lo) of a normalised pair
__device__ __forceinline__ double dd_round(DD a) { return __dadd_rn(a.hi, a.lo); }

// Ziv's rounding test.  (hi, lo) with hi = RN(hi + lo) approximates a value y,
// |y - (hi + lo)| <= err.  y rounds to hi for certain when hi + lo +- err holds
// no midpoint between hi and a neighbour: the neighbour on lo's side is
// ulp(hi) away, ulp(hi) / 2 when that side is toward zero and |hi| is a power
// of two.  (hi = 0 or subnormal: never certain, the caller takes the accurate
// path.)
__device__ __forceinline__ bool rounds_surely(double hi, double lo, double err) {
  const long long b = __double_as_longlong(hi) & 0x7fffffffffffffffll;
  const double ulp = __longlong_as_double(b & 0x7ff0000000000000ll) * 0x1p-52;
  const bool toward_zero = lo != 0.0 && ((lo < 0.0) != (hi < 0.0));
  const double gap = ((b & 0x000fffffffffffffll) == 0 && toward_zero) ? __dmul_rn(0.5, ulp) : ulp;
  return __dadd_ru(fabs(lo), err) < __dmul_rn(0.5, gap);
}

// Error bounds, relative to the result (and absolute, from the argument
// reduction of sin and cos), set above the largest errors measured against
// binary128 on 5 10^6 trajectory arguments per function (log 2^-74.6,
// sin/cos 2^-83.4, acos 2^-84.0): a fast result is kept only when no rounding
// boundary lies within the bound, which sends about 2^-17 (log) and 2^-24
// (sin, cos, acos) of the calls to the accurate paths.
constexpr double kLogFastErr = 0x1p-71;
constexpr double kTrigFastErr = 0x1p-78, kTrigAbsErr = 0x1p-112;
constexpr double kAcosFastErr = 0x1p-78;
__device__ __forceinline__ double rel_err(double v, double rel) { return __dmul_ru(fabs(v), rel); }

// ---------------------------------------------------------------- log
// The entry points are called, not inlined: they are rare next to the spin
// steps, and one copy of each keeps the trajectory code small.  The accurate
// paths are separate calls that most warps never make.

// x = 2^e m, m r = 1 + t exactly (t as double-double), |t| <= 2^-7.
struct LogReduced {
  int e, j;
  DD t;
};
__device__ __forceinline__ LogReduced log_reduce(double x) {
  const long long bits = __double_as_longlong(x);
  int e = (int)((bits >> 52) & 0x7ff) - 1023;
  double m = __longlong_as_double((bits & 0x000fffffffffffffll) | 0x3ff0000000000000ll);  // [1, 2)
  if (m >= 1.5) {
    m = __dmul_rn(m, 0.5);
    e += 1;
  }
  const int j = (int)__dmul_rn(__dsub_rn(m, 0.75), 128.0);  // exact, 0..95
  const DD p = two_prod(m, kLogR[j]);
  return {e, j, two_sum(__dsub_rn(p.hi, 1.0), p.lo)};  // m r - 1, exactly
}
// e ln 2 - log R + l
__device__ __forceinline__ DD log_assemble(const LogReduced& r, DD l) {
  const DD el = dd_add(two_prod((double)r.e, kLn2Hi), two_prod((double)r.e, kLn2Lo));
  const DD lr = {kLogL[r.j][0], kLogL[r.j][1]};
  return dd_add(dd_add(el, lr), l);
}

// log of a positive normal double to ~2^-100: log1p(t) = t sum_n (-1)^(n+1) t^(n-1) / n
// to n = 15 (|t| <= 2^-7) in double-double.
static __device__ __noinline__ double log_accurate(double x) {
  const LogReduced r = log_reduce(x);
  DD q = {kInvN[15][0], kInvN[15][1]};
  for (int n = 14; n >= 1; --n) {
    const DD c = (n & 1) ? DD{kInvN[n][0], kInvN[n][1]} : DD{-kInvN[n][0], -kInvN[n][1]};
    q = dd_add(c, dd_mul(r.t, q));
  }
  return dd_round(log_assemble(r, dd_mul(r.t, q)));
}

// Natural logarithm of a positive normal double, correctly rounded (see the
// file comment); log(1) = 0.
static __device__ __noinline__ double cr_log(double x) {
  const LogReduced r = log_reduce(x);
  const DD t = r.t;
  if (t.hi == 0.0 && r.e == 0 && r.j >= 31 && r.j <= 32) return 0.0;  // x = 1
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
  const DD s = log_assemble(r, l);
  if (rounds_surely(s.hi, s.lo, rel_err(s.hi, kLogFastErr))) return s.hi;
  return log_accurate(x);
}

// ---------------------------------------------------------------- sin, cos
// sin and cos of x, 0 <= |x| < 2^20, as double-double values accurate to
// ~2^-83 relative (absolute ~2^-120 from the reduction).
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
  // s = sh + sl.  z = sh^2 exactly.  sin s = sh + sl + p3 + p5 with
  // p3 = -s^3 / 6 in double-double (s^3 = sh z.hi exactly plus sh z.lo +
  // 3 z.hi sl) and p5 = s^5 / 5! - s^7 / 7! + s^9 / 9! in double;
  // cos s - 1 = cph + cpl with cph = -z.hi / 2 exact and cpl = -z.lo / 2 -
  // sh sl + s^4 / 4! - s^6 / 6! + s^8 / 8!.
  const DD z = two_prod(sh, sh);
  DD s3 = two_prod(sh, z.hi);
  s3.lo = __fma_rn(3.0 * z.hi, sl, __fma_rn(sh, z.lo, s3.lo));
  const DD p3 = dd_mul(s3, {-kSixthHi, -kSixthLo});
  const double p5 = __dmul_rn(__dmul_rn(s3.hi, z.hi),
                             __fma_rn(z.hi, __fma_rn(z.hi, 1.0 / 362880.0, -1.0 / 5040.0), 1.0 / 120.0));
  const double cph = __dmul_rn(-0.5, z.hi);
  const double cpl = __fma_rn(__dmul_rn(z.hi, z.hi),
                              __fma_rn(z.hi, __fma_rn(z.hi, 1.0 / 40320.0, -1.0 / 720.0), 1.0 / 24.0),
                              __fma_rn(-sh, sl, __dmul_rn(-0.5, z.lo)));
  // angle addition with the table at a = j pi / 256: the leading terms (the
  // table value, cos a sh, sin a cph and cos a p3.hi for sin; their
  // counterparts for cos) summed exactly, the rest (below 2^-34 of the
  // result) in double
  const int ja = (int)fabs(jd);
  double sah = kSinA[ja][0], sal = kSinA[ja][1];
  if (jd < 0.0) {
    sah = -sah;
    sal = -sal;
  }
  const double cah = kCosA[ja][0], cal = kCosA[ja][1];
  const double rest_s = __dadd_rn(__dadd_rn(sl, p3.lo), p5);  // sin s - sh - p3.hi
  // sin(a + s) = sin a + cos a (sin s) + sin a (cos s - 1)
  const DD e1 = two_prod(cah, sh), e2 = two_prod(sah, cph), e3 = two_prod(cah, p3.hi);
  const DD h1 = two_sum(sah, e1.hi), h2 = two_sum(h1.hi, e2.hi), h3 = two_sum(h2.hi, e3.hi);
  const double sh3 = __dadd_rn(sh, p3.hi);  // the low table parts multiply sin s to 2^-60
  double ts = __fma_rn(cah, rest_s, __fma_rn(cal, sh3, __fma_rn(sah, cpl, __fma_rn(sal, cph, sal))));
  ts = __dadd_rn(ts, __dadd_rn(__dadd_rn(__dadd_rn(e1.lo, e2.lo), e3.lo), __dadd_rn(__dadd_rn(h1.lo, h2.lo), h3.lo)));
  const DD sr = fast_two_sum(h3.hi, ts);
  // cos(a + s) = cos a - sin a (sin s) + cos a (cos s - 1)
  const DD f1 = two_prod(-sah, sh), f2 = two_prod(cah, cph), f3 = two_prod(-sah, p3.hi);
  const DD g1 = two_sum(cah, f1.hi), g2 = two_sum(g1.hi, f2.hi), g3 = two_sum(g2.hi, f3.hi);
  double tc = __fma_rn(-sah, rest_s, __fma_rn(-sal, sh3, __fma_rn(cah, cpl, __fma_rn(cal, cph, cal))));
  tc = __dadd_rn(tc, __dadd_rn(__dadd_rn(__dadd_rn(f1.lo, f2.lo), f3.lo), __dadd_rn(__dadd_rn(g1.lo, g2.lo), g3.lo)));
  const DD cr = fast_two_sum(g3.hi, tc);
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

// sin and cos of x, 0 <= |x| < 2^20, as double-double values accurate to
// ~2^-100 relative (four-part reduction constants, Taylor series of the
// remainder and the angle addition all in double-double).
static __device__ __noinline__ void sincos_dd_acc(double x, DD& sn, DD& cs) {
  const double k = rint(__dmul_rn(x, kTwoOverPi));
  DD r = two_sum(__fma_rn(-k, kPio2q1, x), __dmul_rn(-k, kPio2q2));
  r = dd_add_d(r, __dmul_rn(-k, kPio2q3));
  r = dd_add(r, dd_neg(two_prod(k, kPio2q4)));
  const double jd = rint(__dmul_rn(r.hi, k256OverPi));
  DD t = two_sum(__fma_rn(-jd, kPio256q1, r.hi), __dmul_rn(-jd, kPio256q2));
  t = dd_add_d(t, r.lo);
  t = dd_add_d(t, __dmul_rn(-jd, kPio256q3));
  t = dd_add(t, dd_neg(two_prod(jd, kPio256q4)));
  // sin t = t sum_k (-1)^k t^2k / (2k+1)!, cos t = sum_k (-1)^k t^2k / (2k)!, k <= 7
  const DD t2 = dd_mul(t, t);
  DD ps = {-kInvFact[15][0], -kInvFact[15][1]};
  DD pc = {kInvFact[16][0], kInvFact[16][1]};
  for (int k = 6; k >= 0; --k) {
    const double sg = (k & 1) ? -1.0 : 1.0;
    ps = dd_add({sg * kInvFact[2 * k + 1][0], sg * kInvFact[2 * k + 1][1]}, dd_mul(t2, ps));
    pc = dd_add({sg * kInvFact[2 * k][0], sg * kInvFact[2 * k][1]}, dd_mul(t2, pc));
  }
  const DD st = dd_mul(t, ps), ct = pc;
  const int ja = (int)fabs(jd);
  DD sa = {kSinA[ja][0], kSinA[ja][1]};
  if (jd < 0.0) sa = dd_neg(sa);
  const DD ca = {kCosA[ja][0], kCosA[ja][1]};
  const DD sr = dd_add(dd_mul(sa, ct), dd_mul(ca, st));           // sin(a + t)
  const DD cr = dd_add(dd_mul(ca, ct), dd_neg(dd_mul(sa, st)));   // cos(a + t)
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

// The correctly rounded double of a fast double-double value of sin or cos
// of x, or of the accurate one when the fast value's rounding is uncertain.
__device__ __forceinline__ bool trig_sure(DD v) {
  return rounds_surely(v.hi, v.lo, __dadd_ru(rel_err(v.hi, kTrigFastErr), kTrigAbsErr));
}
static __device__ __noinline__ void sincos_accurate(double x, double& s, double& c) {
  DD sn, cs;
  sincos_dd_acc(x, sn, cs);
  s = dd_round(sn);
  c = dd_round(cs);
}

// sin and cos of x, 0 <= |x| < 2^20, each correctly rounded (see the file comment).
static __device__ __noinline__ void cr_sincos(double x, double& s, double& c) {
  DD sn, cs;
  sincos_dd(x, sn, cs);
  s = sn.hi;
  c = cs.hi;
  if (!(trig_sure(sn) && trig_sure(cs))) sincos_accurate(x, s, c);
}

// ---------------------------------------------------------------- acos
// acos(x) for x in [0, 1) to ~2^-100: two Newton steps on cos(y) = x in
// double-double from y (a fast estimate), the residual without cancellation
// as in the fast path.
static __device__ __noinline__ double acos_accurate(double x, DD y) {
  for (int it = 0; it < 2; ++it) {
    DD g;
    double sy;
    if (x >= 0.5) {  // g = (1 - x) - 2 sin^2(y / 2); sin(h + l) = sin h + l cos h to ~2^-107
      const DD hy = dd_mul_pow2(y, 0.5);
      DD sn, cs;
      sincos_dd_acc(hy.hi, sn, cs);
      const DD sh = dd_add(sn, dd_mul_d(cs, hy.lo));
      g = dd_add_d(dd_neg(dd_mul_pow2(dd_mul(sh, sh), 2.0)), __dsub_rn(1.0, x));
      sy = __dmul_rn(2.0, __dmul_rn(sh.hi, cs.hi));
    } else {         // g = cos(y) - x; cos(h + l) = cos h - l sin h
      DD sn, cs;
      sincos_dd_acc(y.hi, sn, cs);
      g = dd_add_d(dd_add(cs, dd_neg(dd_mul_d(sn, y.lo))), -x);
      sy = sn.hi;
    }
    y = dd_add_d(y, __ddiv_rn(g.hi, sy));
  }
  return dd_round(y);
}

// y = acos(x) for x in [0, 1], correctly rounded, with sin(y) and cos(y)
// correctly rounded too (a cosine-law reflection needs all three).  CUDA's
// acos gives y0; one Newton step with the double-double sin and cos of y0
// (of y0 / 2 for x >= 1/2) gives y; when y rounds to y0 (most arguments)
// those sin and cos are y's, else they are evaluated again.
static __device__ __noinline__ void cr_acos_sincos(double x, double& y, double& sy, double& cy) {
  const double y0 = acos(x);
  if (x >= 1.0 || x != x) {  // acos(1) = 0 exactly; NaN passes through
    y = y0;
    sy = y0 == 0.0 ? 0.0 : y0;
    cy = y0 == 0.0 ? 1.0 : y0;
    return;
  }
  DD sn, cs;  // sin(y0), cos(y0)
  double g;   // cos(y0) - x
  if (x >= 0.5) {
    DD s2, c2;  // of y0 / 2 (exact halving)
    sincos_dd(__dmul_rn(0.5, y0), s2, c2);
    const DD v = dd_mul_pow2(dd_mul(s2, s2), 2.0);  // 1 - cos(y0) = 2 sin^2(y0 / 2)
    g = dd_round(dd_add_d(dd_neg(v), __dsub_rn(1.0, x)));
    sn = dd_mul_pow2(dd_mul(s2, c2), 2.0);
    cs = dd_add_d(dd_neg(v), 1.0);
  } else {
    sincos_dd(y0, sn, cs);
    g = dd_round(dd_add_d(cs, -x));
  }
  const DD yd = two_sum(y0, __ddiv_rn(g, dd_round(sn)));
  y = yd.hi;
  if (!rounds_surely(yd.hi, yd.lo, rel_err(yd.hi, kAcosFastErr))) y = acos_accurate(x, yd);
  if (y != y0) sincos_dd(y, sn, cs);
  sy = sn.hi;
  cy = cs.hi;
  if (!(trig_sure(sn) && trig_sure(cs))) sincos_accurate(y, sy, cy);
}

static __device__ __noinline__ double cr_acos(double x) {
  double y, sy, cy;
  cr_acos_sincos(x, y, sy, cy);
  return y;
}

// The accurate paths alone (tests): fn 0 log, 1 sin, 2 cos, 3 acos.
static __device__ __noinline__ double cr_accurate_only(int fn, double x) {
  double s, c;
  switch (fn) {
    case 0: return log_accurate(x);
    case 1: sincos_accurate(x, s, c); return s;
    case 2: sincos_accurate(x, s, c); return c;
    default: return (x >= 1.0 || x != x) ? acos(x) : acos_accurate(x, {acos(x), 0.0});
  }
}

}  // namespace crm
}  // namespace st
