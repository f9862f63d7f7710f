// Host build of the device's correctly rounded trajectory functions
// (spin-tracking_gb300/csrc/st_crmath.cuh) for tests: the CUDA intrinsics it
// uses are given their IEEE meaning (round-to-nearest operations, fused
// multiply-add, directed rounding through fesetround), so the same source runs
// on the CPU.  CUDA's acos, the start of the acos Newton step, is the host C
// library's here; the step's error bound covers any start within a few ulps.
//
// For n seeded trajectory arguments per function (the reflection's theta =
// 2 pi u and phi = acos(sqrt u) with the sin and cos of phi; the gas clock's
// log(1 - u) and the Marsaglia polar method's log s), it prints:
//   maxerr <name> <log2 of the largest relative error of the fast double-double value>
//   bound <name> <log2 of the bound the rounding test assumes>
//   wrong <name> <results that differ from the binary128 evaluation rounded once>
//   slow <name> <calls that took the accurate path>
// Build: g++ -O2 -std=c++17 -ffp-contract=off -frounding-math (+ -lquadmath
// where long double is not binary128).
#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>

#if defined(__LDBL_MANT_DIG__) && __LDBL_MANT_DIG__ == 113
typedef long double quad;
static quad q_sin(quad x) { return sinl(x); }
static quad q_cos(quad x) { return cosl(x); }
static quad q_acos(quad x) { return acosl(x); }
static quad q_log(quad x) { return logl(x); }
static double q_log2(quad x) { return (double)log2l(x); }
static quad q_abs(quad x) { return fabsl(x); }
#else
#include <quadmath.h>
typedef __float128 quad;
static quad q_sin(quad x) { return sinq(x); }
static quad q_cos(quad x) { return cosq(x); }
static quad q_acos(quad x) { return acosq(x); }
static quad q_log(quad x) { return logq(x); }
static double q_log2(quad x) { return (double)log2q(x); }
static quad q_abs(quad x) { return fabsq(x); }
#endif

#define __device__
#define __noinline__ __attribute__((noinline))
#define __forceinline__ inline
static inline double __dadd_rn(double a, double b) { return a + b; }
static inline double __dsub_rn(double a, double b) { return a - b; }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __ddiv_rn(double a, double b) { return a / b; }
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
static inline double __dadd_ru(double a, double b) {
  std::fesetround(FE_UPWARD);
  volatile double r = a + b;
  std::fesetround(FE_TONEAREST);
  return r;
}
static inline double __dmul_ru(double a, double b) {
  std::fesetround(FE_UPWARD);
  volatile double r = a * b;
  std::fesetround(FE_TONEAREST);
  return r;
}
static inline long long __double_as_longlong(double x) {
  long long r;
  std::memcpy(&r, &x, 8);
  return r;
}
static inline double __longlong_as_double(long long x) {
  double r;
  std::memcpy(&r, &x, 8);
  return r;
}
using std::acos;
using std::fabs;
using std::rint;
#include "st_crmath.cuh"

using namespace st::crm;

static uint64_t g_state = 0x9E3779B97F4A7C15ull;
static double uniform() {  // xorshift64*, top 53 bits
  g_state ^= g_state >> 12;
  g_state ^= g_state << 25;
  g_state ^= g_state >> 27;
  return (double)((g_state * 0x2545F4914F6CDD1Dull) >> 11) * 0x1p-53;
}

struct Stat {
  const char* name;
  double bound;
  quad maxerr = 0;
  long wrong = 0, slow = 0;
  void err(DD v, quad exact) {
    const quad e = q_abs(((quad)v.hi + (quad)v.lo - exact) / exact);
    if (e > maxerr) maxerr = e;
  }
  void print() const {
    std::printf("maxerr %s %.3f\nbound %s %.3f\nwrong %s %ld\nslow %s %ld\n", name,
                maxerr > 0 ? q_log2(maxerr) : -1000.0, name, std::log2(bound), name, wrong, name, slow);
  }
};

int main(int argc, char** argv) {
  const long n = argc > 1 ? std::atol(argv[1]) : 100000;
  if (argc > 2) g_state = std::strtoull(argv[2], nullptr, 10) | 1ull;
  Stat s_sin{"sin", kTrigFastErr}, s_cos{"cos", kTrigFastErr}, s_acos{"acos", kAcosFastErr},
      s_asin{"sin_acos", kTrigFastErr}, s_acosc{"cos_acos", kTrigFastErr}, s_log{"log", kLogFastErr};
  for (long i = 0; i < n; ++i) {
    // theta = 2 pi u2 of a diffuse reflection
    const double th = (uniform() * 2.0) * 3.141592653589793;
    DD sn, cs;
    sincos_dd(th, sn, cs);
    const quad qs = q_sin(th), qc = q_cos(th);
    if (qs != 0) s_sin.err(sn, qs);
    s_cos.err(cs, qc);
    double s, c;
    if (!cr_sincos_fast(th, s, c)) ++s_sin.slow;
    cr_sincos(th, s, c);
    s_sin.wrong += s != (double)qs;
    s_cos.wrong += c != (double)qc;
    // phi = acos(sqrt u1) with its sin and cos
    const double x = std::sqrt(uniform());
    const double y0 = acos(x);
    DD yd, an, ac;
    acos_newton(x, y0, yd, an, ac);
    const quad qa = q_acos((quad)x);
    s_acos.err(yd, qa);
    const double yr = (double)qa;  // the correctly rounded phi
    sincos_shift(yr - y0, an, ac);
    const quad qsa = q_sin((quad)yr), qca = q_cos((quad)yr);
    s_asin.err(an, qsa);
    s_acosc.err(ac, qca);
    double y, sy, cy;
    if (!cr_acos_sincos_fast(x, y, sy, cy)) ++s_acos.slow;
    cr_acos_sincos(x, y, sy, cy);
    s_acos.wrong += y != yr;
    s_asin.wrong += sy != (double)qsa;
    s_acosc.wrong += cy != (double)qca;
    // the gas clock's log(1 - u) and a Marsaglia pair's log s
    for (int k = 0; k < 2; ++k) {
      double a;
      if (k == 0) {
        a = 1.0 - uniform();
      } else {
        double u, v;
        do {
          u = uniform() * 2.0 - 1.0;
          v = uniform() * 2.0 - 1.0;
          a = u * u + v * v;
        } while (a >= 1.0 || a == 0.0);
      }
      const quad ql = q_log((quad)a);
      double l;
      if (!cr_log_fast(a, l)) ++s_log.slow;
      s_log.wrong += cr_log(a) != (double)ql;
      const LogReduced r = log_reduce(a);
      if (!log_is_one(r)) s_log.err(log_fast_dd(r), ql);
    }
  }
  std::printf("n %ld\n", n);
  for (const Stat* st : {&s_sin, &s_cos, &s_acos, &s_asin, &s_acosc, &s_log}) st->print();
  return 0;
}
