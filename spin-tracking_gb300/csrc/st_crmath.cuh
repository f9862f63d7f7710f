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
//   sin/cos: Cody-Waite reduction by pi/2 with three-part constants (exact
//        products for the arguments used here, |x| < 2^20), then by pi/1024
//        (fast path; table of sin, cos(j pi / 1024) in double-double, Taylor
//        series of the remainder |s| <= pi/2048 in double) or by pi/256 with
//        four-part constants (accurate path; table at j pi / 256, series to
//        s^15 in double-double), angle addition.
//   acos: CUDA's acos as the start y0 and one Newton step on cos(y) = x, whose
//        residual is formed without cancellation: (1 - x) - 2 sin^2(y0 / 2)
//        for x >= 1/2 (1 - x is exact there), cos(y0) - x below; the accurate
//        path repeats the step twice in double-double.  The reflection's sin
//        and cos of the result are the step's sin and cos of y0 carried to y
//        to first order (y - y0 is a few ulps), each with its own rounding
//        test.
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
// 1/x to ~2^-22 (the hardware's approximate reciprocal; a host build of this
// file, for emulation, divides)
__device__ __forceinline__ double rcp_seed(double x) {
#ifdef __CUDA_ARCH__
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  return r;
#else
  return 1.0 / x;
#endif
}
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
// binary128 on 2 10^7 trajectory arguments per function (log 2^-74.6; sin/cos
// 2^-70.2, and 2^-69.5 for the reflection's sin and cos carried from y0 to y;
// the acos Newton step 2^-70.3): a fast result is kept only when no rounding
// boundary lies within the bound, which sends about 2^-17 (log) and 2^-12
// (sin, cos, acos) of the calls to the accurate paths.
constexpr double kLogFastErr = 0x1p-71;
constexpr double kTrigFastErr = 0x1p-66, kTrigAbsErr = 0x1p-112;
constexpr double kAcosFastErr = 0x1p-66;
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

// The fast evaluations are leaf calls that return whether their result is
// certain; the entry points below (and the trajectory's wrappers) call the
// accurate paths only when it is not, so the common call makes no nested call.

// Natural logarithm of a positive normal double: the correctly rounded y and
// true, or false when the fast value's rounding is uncertain; log(1) = 0.
// The fast double-double log of x from its reduction (x != 1).
__device__ __forceinline__ DD log_fast_dd(const LogReduced& r) {
  const DD t = r.t;
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
  return log_assemble(r, l);
}
__device__ __forceinline__ bool log_is_one(const LogReduced& r) {
  return r.t.hi == 0.0 && r.e == 0 && r.j >= 31 && r.j <= 32;
}
static __device__ __noinline__ bool cr_log_fast(double x, double& y) {
  const LogReduced r = log_reduce(x);
  if (log_is_one(r)) {  // x = 1
    y = 0.0;
    return true;
  }
  const DD s = log_fast_dd(r);
  y = s.hi;
  return rounds_surely(s.hi, s.lo, rel_err(s.hi, kLogFastErr));
}

// Natural logarithm of a positive normal double, correctly rounded (see the
// file comment).
static __device__ __noinline__ double cr_log(double x) {
  double y;
  return cr_log_fast(x, y) ? y : log_accurate(x);
}

// ---------------------------------------------------------------- sin, cos
// sin and cos of x, 0 <= |x| < 2^20, as double-double values accurate to
// ~2^-71 relative (absolute ~2^-120 from the reduction): x = k pi/2 + j pi/1024
// + s, |s| <= pi/2048, the Taylor series of sin s - s and cos s - 1 in double
// (their rounding is below 2^-72 of the result at that |s|), and the angle
// addition with the leading product (cos a s for sin, sin a s for cos) exact.
__device__ __forceinline__ void sincos_dd(double x, DD& sn, DD& cs) {
  // x = k pi/2 + r, r as double-double (k * kPio21 and k * kPio22 are exact)
  const double k = rint(__dmul_rn(x, kTwoOverPi));
  const double r1 = __fma_rn(-k, kPio21, x);
  DD r = two_sum(r1, __dmul_rn(-k, kPio22));
  r = dd_add(r, dd_neg(two_prod(k, kPio23)));
  // r = j pi/1024 + s (j * kPio10241 and j * kPio10242 are exact, |j| <= 256)
  const double jd = rint(__dmul_rn(r.hi, k1024OverPi));
  DD t = two_sum(__fma_rn(-jd, kPio10241, r.hi), __dmul_rn(-jd, kPio10242));
  t = dd_add_d(t, r.lo);
  const double sh = t.hi, sl = __fma_rn(-jd, kPio10243, t.lo);
  // sin s - sh = sl - s^3/6 + s^5/120 - s^7/5040; cos s - 1 = -s^2/2 + s^4/24 - s^6/720
  const double z = __dmul_rn(sh, sh);
  const double sp = __dmul_rn(__dmul_rn(sh, z), __fma_rn(z, __fma_rn(z, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0));
  const double cp = __fma_rn(-sh, sl, __dmul_rn(z, __fma_rn(z, __fma_rn(z, -1.0 / 720.0, 1.0 / 24.0), -0.5)));
  const double ss = __dadd_rn(sl, sp);
  const int ja = (int)fabs(jd);
  double sah = kSinB[ja][0], sal = kSinB[ja][1];
  if (jd < 0.0) {
    sah = -sah;
    sal = -sal;
  }
  const double cah = kCosB[ja][0], cal = kCosB[ja][1];
  // sin(a + s) = sin a + cos a sh + [cos a (sin s - sh) + sin a (cos s - 1)]
  const DD m = two_prod(cah, sh);
  const DD hs = two_sum(sah, m.hi);
  const double ts = __dadd_rn(__dadd_rn(m.lo, sal), __fma_rn(cal, sh, __fma_rn(sah, cp, __dmul_rn(cah, ss))));
  const DD sr = fast_two_sum(hs.hi, __dadd_rn(hs.lo, ts));
  // cos(a + s) = cos a - sin a sh + [cos a (cos s - 1) - sin a (sin s - sh)]
  const DD m2 = two_prod(-sah, sh);
  const DD hc = two_sum(cah, m2.hi);
  const double tc = __dadd_rn(__dadd_rn(m2.lo, cal), __fma_rn(-sal, sh, __fma_rn(cah, cp, __dmul_rn(-sah, ss))));
  const DD cr = fast_two_sum(hc.hi, __dadd_rn(hc.lo, tc));
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

// sin and cos of x, 0 <= |x| < 2^20: the correctly rounded pair and true, or
// false when the rounding of either is uncertain.
static __device__ __noinline__ bool cr_sincos_fast(double x, double& s, double& c) {
  DD sn, cs;
  sincos_dd(x, sn, cs);
  s = sn.hi;
  c = cs.hi;
  return trig_sure(sn) && trig_sure(cs);
}

// sin and cos of x, 0 <= |x| < 2^20, each correctly rounded (see the file comment).
static __device__ __noinline__ void cr_sincos(double x, double& s, double& c) {
  if (!cr_sincos_fast(x, s, c)) sincos_accurate(x, s, c);
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

// One Newton step on cos(y) = x from y0 (CUDA's acos, x in [0, 1)): yd as
// double-double, with the double-double sin and cos of y0.  For x >= 1/2 the
// residual is (1 - x) - 2 sin^2(y0 / 2) (exact halving, no cancellation).
// The step takes the sin and cos of acos_newton_arg(x, y0) (y0 / 2 or y0),
// sa and ca, from its caller.
__device__ __forceinline__ double acos_newton_arg(double x, double y0) { return x >= 0.5 ? __dmul_rn(0.5, y0) : y0; }
__device__ __forceinline__ void acos_newton_given(double x, double y0, DD sa, DD ca, DD& yd, DD& sn, DD& cs) {
  double g;  // cos(y0) - x
  if (x >= 0.5) {
    const DD v = dd_mul_pow2(dd_mul(sa, sa), 2.0);  // 1 - cos(y0)
    g = dd_round(dd_add_d(dd_neg(v), __dsub_rn(1.0, x)));
    sn = dd_mul_pow2(dd_mul(sa, ca), 2.0);
    cs = dd_add_d(dd_neg(v), 1.0);
  } else {
    sn = sa;
    cs = ca;
    g = dd_round(dd_add_d(cs, -x));
  }
  // the correction g / sin(y0) is a few ulps of y0, so a reciprocal to 2^-44
  // (hardware seed and one Newton step) leaves it exact to ~2^-96 of y0
  const double q = dd_round(sn);
  double r = rcp_seed(q);
  r = __fma_rn(r, __fma_rn(-q, r, 1.0), r);
  yd = two_sum(y0, __dmul_rn(g, r));
}
__device__ __forceinline__ void acos_newton(double x, double y0, DD& yd, DD& sn, DD& cs) {
  DD sa, ca;
  sincos_dd(acos_newton_arg(x, y0), sa, ca);
  acos_newton_given(x, y0, sa, ca, yd, sn, cs);
}
// sin and cos of y0 + d from those of y0, for d a few ulps of y0 (exact):
// sin y0 + d cos y0 and cos y0 - d sin y0, to d^2 / 2 < 2^-100 of the result.
__device__ __forceinline__ void sincos_shift(double d, DD& sn, DD& cs) {
  if (d == 0.0) return;
  const double s0 = sn.hi;
  sn = dd_add_d(sn, __dmul_rn(d, cs.hi));
  cs = dd_add_d(cs, __dmul_rn(-d, s0));
}

// y = acos(x) for x in [0, 1], correctly rounded, with sin(y) and cos(y)
// correctly rounded too (a cosine-law reflection needs all three): a Newton
// step from CUDA's acos, the sin and cos of that y0 carried to y to first
// order, each value kept when its rounding is certain (Ziv's test) and
// evaluated by the accurate paths otherwise.  The _fast form returns false
// instead of taking an accurate path.
// The fast form from y0 = acos(x) and the sin and cos of acos_newton_arg(x,
// y0), for callers that evaluate those themselves.
__device__ __forceinline__ bool acos_sincos_given(double x, double y0, DD sa, DD ca, double& y, double& sy,
                                                  double& cy) {
  if (x >= 1.0 || x != x) {  // acos(1) = 0 exactly; NaN passes through
    y = y0;
    sy = y0 == 0.0 ? 0.0 : y0;
    cy = y0 == 0.0 ? 1.0 : y0;
    return true;
  }
  DD yd, sn, cs;
  acos_newton_given(x, y0, sa, ca, yd, sn, cs);
  y = yd.hi;
  sincos_shift(__dsub_rn(y, y0), sn, cs);
  sy = sn.hi;
  cy = cs.hi;
  return rounds_surely(yd.hi, yd.lo, rel_err(yd.hi, kAcosFastErr)) && trig_sure(sn) && trig_sure(cs);
}
static __device__ __noinline__ bool cr_acos_sincos_fast(double x, double& y, double& sy, double& cy) {
  const double y0 = acos(x);
  DD sa{0.0, 0.0}, ca{1.0, 0.0};
  if (x < 1.0) sincos_dd(acos_newton_arg(x, y0), sa, ca);  // NaN and 1 need none
  return acos_sincos_given(x, y0, sa, ca, y, sy, cy);
}

static __device__ __noinline__ void cr_acos_sincos(double x, double& y, double& sy, double& cy) {
  const double y0 = acos(x);
  if (x >= 1.0 || x != x) {  // acos(1) = 0 exactly; NaN passes through
    y = y0;
    sy = y0 == 0.0 ? 0.0 : y0;
    cy = y0 == 0.0 ? 1.0 : y0;
    return;
  }
  DD yd, sn, cs;
  acos_newton(x, y0, yd, sn, cs);
  y = yd.hi;
  if (!rounds_surely(yd.hi, yd.lo, rel_err(yd.hi, kAcosFastErr))) y = acos_accurate(x, yd);
  sincos_shift(__dsub_rn(y, y0), sn, cs);
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
