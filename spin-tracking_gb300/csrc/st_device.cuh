// Device building blocks of the hot path: the RNG, the ballistic trajectory
// events, the field polynomial and single step attempts of DOP853, RK45 and
// the integrator types 2-5 (Magnus CFET8, RK45 / RKF45 with quaternions, RKF45).
//
// Two arithmetic regimes:
//  * Trajectory and RNG code reproduces the reference's doubles bit for bit
//    (same operation order, no FMA contraction: every add/mul/div/sqrt is an
//    explicit round-to-nearest intrinsic), so event times, bounce/collision
//    counts and RNG draws match the CPU build exactly.  Its log, acos, cos and
//    sin are the correctly rounded ones of st_crmath.cuh (equal to the host C
//    library's wherever those are correctly rounded), or CUDA's with
//    ST_TRAJ_CORRECTLY_ROUNDED 0 (st_fields.cuh).
//  * The spin steppers are restated for the FP64 pipe: FMA-contracted stage
//    sums, the field as a polynomial in segment time, reciprocal-form error
//    weights and step controller.  Results agree with the reference to the
//    integration tolerance, not bit for bit.
#pragma once

#include <float.h>
#include <stdint.h>
#include "st_internal.h"
#include "st_fields.cuh"
#include "st_tableau.h"
#include "st_crmath.cuh"

namespace st {
// The trajectory's transcendental functions (ST_TRAJ_CORRECTLY_ROUNDED, st_fields.cuh).
__device__ __forceinline__ double traj_log(double x) {
#if ST_TRAJ_CORRECTLY_ROUNDED
  double y;
  return crm::cr_log_fast(x, y) ? y : crm::log_accurate(x);
#else
  return log(x);
#endif
}
// acos(x) and the sin and cos of the result
__device__ __forceinline__ void traj_acos_sincos(double x, double& y, double& sy, double& cy) {
#if ST_TRAJ_CORRECTLY_ROUNDED
  if (!crm::cr_acos_sincos_fast(x, y, sy, cy)) crm::cr_acos_sincos(x, y, sy, cy);
#else
  y = acos(x);
  sy = sin(y);
  cy = cos(y);
#endif
}
__device__ __forceinline__ void traj_sincos(double x, double& s, double& c) {
#if ST_TRAJ_CORRECTLY_ROUNDED
  if (!crm::cr_sincos_fast(x, s, c)) crm::sincos_accurate(x, s, c);
#else
  s = sin(x);
  c = cos(x);
#endif
}
}  // namespace st

namespace st {

// ------------------------------------------------------------------ exact ops
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double xsqrt(double a) { return __dsqrt_rn(a); }
// sgn with sgn(0) = +1 (src/particle.cpp:24-31)
__device__ __forceinline__ double sgn1(double v) { return v < 0.0 ? -1.0 : 1.0; }
// std::min / std::max argument conventions
__device__ __forceinline__ double std_min(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double std_max(double a, double b) { return (a < b) ? b : a; }
// min_d / max_d (src/integrator.cpp:25-33)
__device__ __forceinline__ double min_d(double a, double b) { return (a < b) ? a : b; }
__device__ __forceinline__ double max_d(double a, double b) { return (a > b) ? a : b; }

// ------------------------------------------------------------ fast FP64 roots
// Approximate hardware seeds (PTX rcp.approx / rsqrt.approx, ~2^-22 relative)
// refined by FMA Newton steps on the FP64 pipe.
__device__ __forceinline__ double rcp_seed(double x) {
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  return r;
}
__device__ __forceinline__ double rsqrt_seed(double x) {
  double r;
  asm("rsqrt.approx.f64 %0, %1;" : "=d"(r) : "d"(x));
  return r;
}
// 1/x to full double precision for finite nonzero x; 0 and inf pass through.
__device__ __forceinline__ double rcp_full(double x) {
  const double r = rcp_seed(x);
  const double e = fma(-x, r, 1.0);
  const double r2 = fma(r, fma(e, e, e), r);  // third-order correction
  return (e == e) ? r2 : r;
}
// 1/sqrt(x) to full double precision for finite positive x.
__device__ __forceinline__ double rsqrt_full(double x) {
  const double y = rsqrt_seed(x);
  const double e = fma(-x * y, y, 1.0);
  const double y2 = fma(y * e, fma(0.375, e, 0.5), y);  // third-order correction
  return (e == e) ? y2 : y;
}
// x^(-1/8) for 1e-300 < x < 1e300: chained rsqrt seeds, two Newton steps on
// r^8 x = 1.
__device__ __forceinline__ double rroot8(double x) {
  double r = rsqrt_seed(rsqrt_seed(rsqrt_seed(x)));
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const double r2 = r * r, r4 = r2 * r2;
    const double u = (r4 * r4) * x;
    r = fma(r, fma(u, -0.125, 0.125), r);
  }
  return r;
}

// ------------------------------------------------------------------------ RNG
// Reference rngState (include/particle.h:52-59) and its generator.
struct Rng {
  uint64_t x, y, z, w;
  double spare;
  bool has;
};

// xoshiro256+ as the reference implements it (src/particle.cpp:59-70): the
// last word is re-derived from the third, not rotated in place.
__device__ __forceinline__ uint64_t rng_next(Rng& r) {
  const uint64_t out = r.x + r.z;
  const uint64_t t = r.y << 17;
  r.z ^= r.x;
  r.w ^= r.y;
  r.y ^= r.z;
  r.x ^= r.w;
  r.z ^= t;
  r.w = (r.z << 45) | (r.z >> 19);
  return out;
}
// top 53 bits scaled by 2^-53 (exact), src/particle.cpp:72-83
__device__ __forceinline__ double rng_uniform(Rng& r) { return xmul((double)(rng_next(r) >> 11), 0x1.0p-53); }

// The uniform pairs of the Marsaglia polar method until 0 < s = u^2 + v^2 < 1,
// and the factor sqrt(-2 log s / s) from log s.
__device__ __forceinline__ void marsaglia_draw(Rng& r, double& u, double& v, double& s) {
  do {
    u = xadd(xmul(rng_uniform(r), 2.0), -1.0);
    v = xadd(xmul(rng_uniform(r), 2.0), -1.0);
    s = xadd(xmul(u, u), xmul(v, v));
  } while (s >= 1.0 || s == 0.0);
}
__device__ __forceinline__ double marsaglia_factor(double s, double log_s) { return xsqrt(xdiv(xmul(-2.0, log_s), s)); }

// Marsaglia polar normal with cached spare (src/particle.cpp:89-107).
__device__ __forceinline__ double rng_normal(Rng& r, double mean, double sd) {
  if (r.has) {
    r.has = false;
    return xadd(xmul(r.spare, sd), mean);
  }
  double u, v, s;
  marsaglia_draw(r, u, v, s);
  const double f = marsaglia_factor(s, traj_log(s));
  r.spare = xmul(v, f);
  r.has = true;
  return xadd(mean, xmul(xmul(sd, u), f));
}
__device__ __forceinline__ double rng_exponential(Rng& r, double tc) {
  return xmul(-tc, traj_log(xsub(1.0, rng_uniform(r))));
}

// Seeding of initParticlesCPU (src/particle.cpp:648-663): splitmix64 of the
// 32-bit sum seed + ipart, two outputs split into 32-bit halves, three
// discarded draws.
__device__ __forceinline__ uint64_t splitmix_next(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ Rng rng_seed(unsigned int seed, unsigned int ipart) {
  uint64_t s = (uint64_t)(uint32_t)(seed + ipart);
  Rng r;
  const uint64_t a = splitmix_next(s);
  r.x = (uint32_t)a;
  r.y = (uint32_t)(a >> 32);
  const uint64_t b = splitmix_next(s);
  r.z = (uint32_t)b;
  r.w = (uint32_t)(b >> 32);
  r.spare = 0.0;
  r.has = false;
  rng_next(r);
  rng_next(r);
  rng_next(r);
  return r;
}

// ------------------------------------------------------------ particle state
struct PState {
  double t, px, py, pz, vx, vy, vz, Sx, Sy, Sz, h, next_gas;
  Rng rng;
  uint64_t n_coll, n_bounce, n_steps;
  int fail;
  int turns;  // precession turns about x (see count_turn)
  bool stop;
  char coll, wall;
};

__device__ __forceinline__ PState load_state(const DeviceState& s, int64_t i) {
  PState p;
  p.t = s.t[i];
  p.px = s.px[i]; p.py = s.py[i]; p.pz = s.pz[i];
  p.vx = s.vx[i]; p.vy = s.vy[i]; p.vz = s.vz[i];
  p.Sx = s.Sx[i]; p.Sy = s.Sy[i]; p.Sz = s.Sz[i];
  p.h = s.h[i];
  p.next_gas = s.next_gas[i];
  p.rng.x = s.rx[i]; p.rng.y = s.ry[i]; p.rng.z = s.rz[i]; p.rng.w = s.rw[i];
  p.rng.spare = s.rspare[i];
  p.rng.has = s.rhas[i] != 0;
  p.n_coll = s.n_coll[i]; p.n_bounce = s.n_bounce[i]; p.n_steps = s.n_steps[i];
  p.fail = s.fail[i];
  p.turns = s.turns[i];
  p.stop = s.stop[i] != 0;
  p.coll = (char)s.coll[i];
  p.wall = (char)s.wall[i];
  return p;
}

__device__ __forceinline__ void store_state(const DeviceState& s, int64_t i, const PState& p) {
  s.t[i] = p.t;
  s.px[i] = p.px; s.py[i] = p.py; s.pz[i] = p.pz;
  s.vx[i] = p.vx; s.vy[i] = p.vy; s.vz[i] = p.vz;
  s.Sx[i] = p.Sx; s.Sy[i] = p.Sy; s.Sz[i] = p.Sz;
  s.h[i] = p.h;
  s.next_gas[i] = p.next_gas;
  s.rx[i] = p.rng.x; s.ry[i] = p.rng.y; s.rz[i] = p.rng.z; s.rw[i] = p.rng.w;
  s.rspare[i] = p.rng.spare;
  s.rhas[i] = p.rng.has ? 1 : 0;
  s.n_coll[i] = p.n_coll; s.n_bounce[i] = p.n_bounce; s.n_steps[i] = p.n_steps;
  s.fail[i] = p.fail;
  s.turns[i] = p.turns;
  s.stop[i] = p.stop ? 1 : 0;
  s.coll[i] = (uint8_t)p.coll;
  s.wall[i] = (uint8_t)p.wall;
}

// initParticlesCPU for one particle (src/particle.cpp:646-708).
__device__ inline PState init_particle(const SetParams& P, unsigned int ipart) {
  PState p;
  Rng r = rng_seed(P.seed, ipart);
  p.px = xsub(xmul(rng_uniform(r), P.Lx), P.Lx / 2.0);
  p.py = xsub(xmul(rng_uniform(r), P.Ly), P.Ly / 2.0);
  p.pz = xsub(xmul(rng_uniform(r), P.Lz), P.Lz / 2.0);
  p.next_gas = P.gas ? rng_exponential(r, P.tc) : DBL_MAX;
  p.vx = p.vy = p.vz = 0.0;
  if (P.dist == 'C') {
    // the CPU build draws three normals even for V == 0 (src/particle.cpp:677-684)
    const double dx = rng_normal(r, 0.0, 1.0);
    const double dy = rng_normal(r, 0.0, 1.0);
    const double dz = rng_normal(r, 0.0, 1.0);
    const double nrm = xsqrt(xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz)));
    p.vx = xdiv(xmul(dx, P.V), nrm);
    p.vy = xdiv(xmul(dy, P.V), nrm);
    p.vz = xdiv(xmul(dz, P.V), nrm);
  } else if (P.dist == 'M') {
    p.vx = xmul(rng_normal(r, 0.0, 1.0), P.sqrtKT_m);
    p.vy = xmul(rng_normal(r, 0.0, 1.0), P.sqrtKT_m);
    p.vz = xmul(rng_normal(r, 0.0, 1.0), P.sqrtKT_m);
  }
  p.rng = r;
  p.Sx = P.yi_x; p.Sy = P.yi_y; p.Sz = P.yi_z;
  p.t = P.t0;
  p.h = P.h0;
  p.stop = false;
  p.coll = 'W';
  p.wall = 0;
  p.fail = 0;
  p.turns = 0;
  p.n_coll = p.n_bounce = p.n_steps = 0;
  return p;
}

// Start of the current ballistic segment (t_old, pos_old, v_old).
struct SegStart {
  double t, px, py, pz, vx, vy, vz;
};

// A trajectory event whose draws were taken but whose logarithms, sines and
// cosines are not yet computed (traj_event<true>): a cosine-law diffuse
// reflection, or a gas collision with a Maxwell-Boltzmann velocity redraw.
//   reflection: x[0] = sqrt(u1), x[1] = theta = 2 pi u2, x[2] = |v| at the wall
//   gas:        x[0] = 1 - u of the gas clock's exponential draw, then the
//               Marsaglia pairs drawn for the three velocity normals, (u, v, s)
//               in x[1..3] and x[4..6]: one pair when the first normal is the
//               cached spare (spare_first), two otherwise
struct EventDefer {
  double x[7];
  char wall;
  bool pending, gas, spare_first;
};

// New velocity of a cosine-law diffuse reflection off wall w from the sin and
// cos of phi = acos(sqrt u1) and of theta = 2 pi u2 (src/particle.cpp:309-328).
__device__ __forceinline__ void diffuse_apply(PState& p, double sp, double cp, double stt, double ct, double speed,
                                              char w) {
  if (w == 'x') {
    p.vx = xmul(xmul(xmul(-1.0, sgn1(p.vx)), speed), cp);
    p.vy = xmul(xmul(-speed, sp), ct);
    p.vz = xmul(xmul(speed, sp), stt);
  } else if (w == 'y') {
    p.vx = xmul(xmul(speed, sp), ct);
    p.vy = xmul(xmul(xmul(-1.0, sgn1(p.vy)), speed), cp);
    p.vz = xmul(xmul(speed, sp), stt);
  } else {
    p.vx = xmul(xmul(speed, sp), ct);
    p.vy = xmul(xmul(speed, sp), stt);
    p.vz = xmul(xmul(xmul(-1.0, sgn1(p.vz)), speed), cp);
  }
}

// New velocity of a cosine-law diffuse reflection off wall w (src/particle.cpp:309-328).
__device__ __forceinline__ void diffuse_velocity(PState& p, double su, double theta, double speed, char w) {
  double phi, cp, sp, ct, stt;
  traj_acos_sincos(su, phi, sp, cp);
  traj_sincos(theta, stt, ct);
  diffuse_apply(p, sp, cp, stt, ct, speed, w);
}

// Position of the k-th set bit of m, counting from 0 (k < popc(m)).
__device__ __forceinline__ int nth_set_bit(unsigned m, int k) {
  int p = 0;
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const int c = __popc(m & ((1u << s) - 1u));
    if (k >= c) {
      k -= c;
      m >>= s;
      p += s;
    }
  }
  return p;
}

// The rest of a deferred gas collision from the logarithms of its draws
// (log_a of the gas clock's 1 - u, log_s0 and log_s1 of the Marsaglia pairs):
// the gas clock as rng_exponential advances it, the three normals and the
// cached spare as three rng_normal calls leave them, the Maxwell-Boltzmann
// velocity (src/particle.cpp:117-119, 89-111, 373-380).
__device__ __forceinline__ void gas_finish(PState& p, const SetParams& P, const EventDefer& dd, double log_a,
                                           double log_s0, double log_s1) {
  p.next_gas = xadd(p.next_gas, xmul(-P.tc, log_a));
  const double f0 = marsaglia_factor(dd.x[3], log_s0);
  const double pair0 = xadd(0.0, xmul(xmul(1.0, dd.x[1]), f0));
  const double spare0 = xmul(dd.x[2], f0);
  double n1, n2, n3;
  if (dd.spare_first) {
    n1 = xadd(xmul(p.rng.spare, 1.0), 0.0);
    n2 = pair0;
    n3 = xadd(xmul(spare0, 1.0), 0.0);
    p.rng.spare = spare0;
  } else {
    const double f1 = marsaglia_factor(dd.x[6], log_s1);
    n1 = pair0;
    n2 = xadd(xmul(spare0, 1.0), 0.0);
    n3 = xadd(0.0, xmul(xmul(1.0, dd.x[4]), f1));
    p.rng.spare = xmul(dd.x[5], f1);
  }
  p.vx = xmul(n1, P.sqrtKT_m);
  p.vy = xmul(n2, P.sqrtKT_m);
  p.vz = xmul(n3, P.sqrtKT_m);
}

// The deferred events of a warp, lanes `pend`, computed by all 32 lanes
// together (the warp must be converged).  A diffuse reflection needs the sin
// and cos of two angles (the argument of its acos Newton step and theta), a
// gas collision the logarithms of up to three of its draws.  Those
// evaluations are dealt out one per lane per pass (one pass for up to 16
// reflections, another for up to 10 gas collisions) instead of running one
// after the other on each pending lane; each pending lane then finishes its
// own event from the shuffled results.  Every value is computed by the code of
// the per-lane path (diffuse_velocity, rng_exponential, rng_normal), so the
// results are the same bit for bit.
template <bool GAS>
__device__ __forceinline__ void deferred_events_warp(PState& p, const SetParams& P, EventDefer& dd, unsigned pend,
                                                     int lane) {
#if ST_TRAJ_CORRECTLY_ROUNDED
  const unsigned FULL = 0xffffffffu;
  const unsigned below = (1u << lane) - 1u;
  const unsigned refl = GAS ? __ballot_sync(FULL, dd.pending && !dd.gas) : pend;
  if (refl) {
    const int np = __popc(refl);
    const bool mine = dd.pending && !dd.gas;
    const double x = dd.x[0];
    double y0 = 0.0, arg_a = 0.0;
    if (mine) {
      y0 = acos(x);
      arg_a = x < 1.0 ? crm::acos_newton_arg(x, y0) : 0.0;  // NaN and 1 use none
    }
    const int rank = __popc(refl & below);
    crm::DD sa{0.0, 0.0}, ca{1.0, 0.0}, st{0.0, 0.0}, ct{1.0, 0.0};
    for (int base = 0; base < 2 * np; base += 32) {
      // job j = base + lane: the Newton argument of reflection j (j < np) or
      // the theta of reflection j - np
      const int j = base + lane;
      const int src = nth_set_bit(refl, min(j < np ? j : j - np, np - 1));
      const double a1 = __shfl_sync(FULL, arg_a, src), a2 = __shfl_sync(FULL, dd.x[1], src);
      crm::DD sn, cs;
      crm::sincos_dd(j < np ? a1 : a2, sn, cs);
      // the reflection of rank r takes jobs r and np + r
      const int ja = rank - base, jb = np + rank - base;
      const double v0 = __shfl_sync(FULL, sn.hi, ja & 31), v1 = __shfl_sync(FULL, sn.lo, ja & 31);
      const double v2 = __shfl_sync(FULL, cs.hi, ja & 31), v3 = __shfl_sync(FULL, cs.lo, ja & 31);
      const double w0 = __shfl_sync(FULL, sn.hi, jb & 31), w1 = __shfl_sync(FULL, sn.lo, jb & 31);
      const double w2 = __shfl_sync(FULL, cs.hi, jb & 31), w3 = __shfl_sync(FULL, cs.lo, jb & 31);
      if (ja >= 0 && ja < 32) {
        sa = {v0, v1};
        ca = {v2, v3};
      }
      if (jb >= 0 && jb < 32) {
        st = {w0, w1};
        ct = {w2, w3};
      }
    }
    if (mine) {
      double phi, sp, cp;
      if (!crm::acos_sincos_given(x, y0, sa, ca, phi, sp, cp)) crm::cr_acos_sincos(x, phi, sp, cp);
      double stt = st.hi, ctt = ct.hi;
      if (!(crm::trig_sure(st) && crm::trig_sure(ct))) crm::sincos_accurate(dd.x[1], stt, ctt);
      diffuse_apply(p, sp, cp, stt, ctt, dd.x[2], dd.wall);
      dd.pending = false;
    }
  }
  if (GAS) {
    const unsigned gm = pend & ~refl;
    if (gm) {
      const int ng = __popc(gm);
      const bool mine = dd.pending && dd.gas;
      const double third = dd.spare_first ? 1.0 : dd.x[6];  // log 1 = 0 fills the unused job
      const int rank = __popc(gm & below);
      double l0 = 0.0, l1 = 0.0, l2 = 0.0;
      for (int base = 0; base < 3 * ng; base += 32) {
        // job j = base + lane: draw j % 3 (1 - u, s of pair 0, s of pair 1)
        // of gas collision j / 3
        const int j = base + lane;
        const int q = min(j / 3, ng - 1), k = j - 3 * (j / 3);
        const int src = nth_set_bit(gm, q);
        const double a0 = __shfl_sync(FULL, dd.x[0], src), a1 = __shfl_sync(FULL, dd.x[3], src);
        const double a2 = __shfl_sync(FULL, third, src);
        const double arg = k == 0 ? a0 : (k == 1 ? a1 : a2);
        double y;
        if (!crm::cr_log_fast(arg, y)) y = crm::log_accurate(arg);
        // the collision of rank r takes jobs 3r, 3r + 1, 3r + 2
        const int jr = 3 * rank - base;
        const double r0 = __shfl_sync(FULL, y, jr & 31), r1 = __shfl_sync(FULL, y, (jr + 1) & 31);
        const double r2 = __shfl_sync(FULL, y, (jr + 2) & 31);
        if (jr >= 0 && jr < 32) l0 = r0;
        if (jr + 1 >= 0 && jr + 1 < 32) l1 = r1;
        if (jr + 2 >= 0 && jr + 2 < 32) l2 = r2;
      }
      if (mine) {
        gas_finish(p, P, dd, l0, l1, l2);
        dd.pending = false;
        dd.gas = false;
      }
    }
  }
#else
  if (dd.pending) {
    if (GAS && dd.gas)
      gas_finish(p, P, dd, traj_log(dd.x[0]), traj_log(dd.x[3]), dd.spare_first ? 0.0 : traj_log(dd.x[6]));
    else
      diffuse_velocity(p, dd.x[0], dd.x[1], dd.x[2], dd.wall);
    dd.pending = false;
    dd.gas = false;
  }
#endif
}

// One trajectory event: calc_next_collision_time, update_position_and_velocity
// and sanity_check (src/particle.cpp:121-444).  Returns `finished` (the window
// end tf was reached).  Fills the segment start.
//
// DEFER: a diffuse reflection's draws are taken here (the RNG sequence is
// unchanged) but its velocity is left to deferred_events_warp, called later by
// the trajectory-ahead kernel for many lanes at once.  The sanity check then
// sees the velocity before the reflection; that gives the same outcome: the
// reflected velocity is |v| times sines and cosines that are finite and, for
// the draws possible here, non-zero except cos(phi) at u1 = 0, so it is NaN
// or infinite only when the velocity before it already was, which fails the
// same check (NaN) or the position check before it (infinite).  A gas
// collision with a Maxwell-Boltzmann redraw is deferred the same way: its
// uniform draws are taken here in the reference's order, the logarithms (of
// the gas clock and of the Marsaglia pairs) later.  Its new velocity is the
// product of finite normals and a finite sqrt(kT/m), so the NaN check gives the
// outcome it gives on the velocity before the collision (which it also tests).
//
// GAS = false: compiled for launches in which no parameter set has gas
// collisions.  Their gas clock is DBL_MAX and never moves, so the gas
// collision is never the next event: either the wall time is finite and
// smaller, or it is infinite and the step ends at the maxPosStep / window
// limit either way.
template <bool DEFER = false, bool GAS = true>
__device__ __forceinline__ bool traj_event(PState& p, const SetParams& P, double tf, SegStart& s0,
                                           EventDefer* dd = nullptr) {
  const double G = kGravity;
  const double hLx = P.Lx / 2.0, hLy = P.Ly / 2.0, hLz = P.Lz / 2.0;
  double dtx, dty, dtz;
  // ---- time to the next wall (calc_next_collision_time)
  if (P.gravity) {
    const double dx = xsub(sgn1(p.vx) < 0.0 ? -hLx : hLx, p.px);
    const double dz = xsub(sgn1(p.vz) < 0.0 ? -hLz : hLz, p.pz);
    dtx = xdiv(dx, p.vx);
    dtz = xdiv(dz, p.vz);
    const double y2 = xmul(p.vy, p.vy);
    // Moving down meets the floor; moving up meets the ceiling unless the apex
    // is below it (then rise and fall to the floor).  Floor and ceiling share
    // one root pair: the reference's ceiling roots (-vy + sq)/G, (-vy - sq)/G
    // are bit for bit its floor roots (sq - vy)/G, -(sq + vy)/G in swapped
    // order (IEEE addition commutes, negation is exact), and min(|r1|, |r2|)
    // does not depend on the order (both roots are NaN together), so both
    // branches run the same sqrt and divisions, once.
    bool apex = false;
    double arg = 0.0;
    if (sgn1(p.vy) <= 0.0) {
      const double dy = xadd(p.py, xmul(P.Ly, 0.5));
      arg = xadd(xmul(-2.0 * G, dy), y2);
    } else {
      const double top = xadd(xdiv(xmul(-0.5, y2), G), p.py);
      apex = top < xmul(0.5, P.Ly);
      arg = xsub(y2, xmul(2.0 * G, xsub(p.py, xmul(0.5, P.Ly))));
    }
    if (!apex) {
      const double sq = xsqrt(arg);
      const double r1 = xdiv(-xadd(sq, p.vy), G);
      const double r2 = xdiv(xsub(sq, p.vy), G);
      dty = std_min(fabs(r1), fabs(r2));
    } else {
      const double t1 = xdiv(-p.vy, G);
      const double ap = xadd(xadd(p.py, xmul(p.vy, t1)), xmul(xmul(0.5 * G, t1), t1));
      const double t2 = xsqrt(xdiv(xmul(xsub(xmul(-0.5, P.Ly), ap), 2.0), G));
      dty = xadd(t1, t2);
    }
    if (dtx < 1e-16 || isnan(dtx))  // only the first offending axis is replaced
      dtx = 1e6;
    else if (dty < 1e-16 || isnan(dty))
      dty = 1e6;
    else if (dtz < 1e-16 || isnan(dtz))
      dtz = 1e6;
  } else {
    dtx = xdiv(xsub(sgn1(p.vx) < 0.0 ? -hLx : hLx, p.px), p.vx);
    dty = xdiv(xsub(sgn1(p.vy) < 0.0 ? -hLy : hLy, p.py), p.vy);
    dtz = xdiv(xsub(sgn1(p.vz) < 0.0 ? -hLz : hLz, p.pz), p.vz);
    if (dtx < 1e-16)
      dtx = 1e6;
    else if (dty < 1e-16)
      dty = 1e6;
    else if (dtz < 1e-16)
      dtz = 1e6;
  }
  double tb = __longlong_as_double(0x7ff8000000000000ll);  // unset when every comparison fails (NaN input)
  if (dtx < dty && dtx < dtz) {
    tb = dtx; p.wall = 'x';
  } else if (dty < dtx && dty < dtz) {
    tb = dty; p.wall = 'y';
  } else if (dtz < dtx && dtz < dty) {
    tb = dtz; p.wall = 'z';
  } else if (dtx == dty && dtx == dtz) {
    tb = dtx; p.wall = 'a';  // corner
  } else if (dtx == dty) {
    tb = dtx; p.wall = 'b';  // x-y edge
  } else if (dtx == dtz) {
    tb = dtx; p.wall = 'c';  // x-z edge
  } else if (dty == dtz) {
    tb = dty; p.wall = 'd';  // y-z edge
  }
  // ---- gas collision, wall, window end or maxPosStep
  bool gas_next = false;
  double to_col = tb;
  const double to_gas = GAS ? xsub(p.next_gas, p.t) : 0.0;
  if (!GAS) {
    // no gas collisions in this launch
  } else if (to_gas < tb) {
    gas_next = true;
    to_col = to_gas;
  } else if (to_gas == tb) {  // tie: the wall wins and the gas clock is redrawn
    p.next_gas = xadd(p.next_gas, rng_exponential(p.rng, P.tc));
    to_col = to_gas;
    gas_next = false;
  } else {
    gas_next = false;
    to_col = tb;
  }
  const double left = xsub(tf, p.t);
  const bool window_end = left <= P.maxPosStep;
  const double to_free = window_end ? left : P.maxPosStep;
  bool finished = false;
  double dt;
  if (to_col <= to_free) {
    dt = to_col;
    if (gas_next) {
      p.coll = 'G';
      p.n_coll += 1;
      if (DEFER && P.dist == 'M' && isfinite(P.sqrtKT_m)) {
        dd->x[0] = xsub(1.0, rng_uniform(p.rng));  // rng_exponential's draw; its log later
        dd->gas = true;
      } else {
        p.next_gas = xadd(p.next_gas, rng_exponential(p.rng, P.tc));
      }
    } else {
      p.n_bounce += 1;
      p.coll = 'W';
    }
    if (to_col == to_free && window_end) finished = true;
  } else {
    p.coll = 'N';
    dt = to_free;
    if (window_end) finished = true;
  }
  // ---- ballistic move (update_position_and_velocity)
  s0.t = p.t;
  s0.px = p.px; s0.py = p.py; s0.pz = p.pz;
  s0.vx = p.vx; s0.vy = p.vy; s0.vz = p.vz;
  p.t = xadd(p.t, dt);
  const double ay = P.gravity ? G : 0.0;
  const double hax = xmul(xmul(0.5 * 0.0, dt), dt);
  const double hay = xmul(xmul(0.5 * ay, dt), dt);
  p.px = xadd(xadd(s0.px, xmul(s0.vx, dt)), hax);
  p.py = xadd(xadd(s0.py, xmul(s0.vy, dt)), hay);
  p.pz = xadd(xadd(s0.pz, xmul(s0.vz, dt)), hax);
  p.vx = xadd(p.vx, xmul(0.0, dt));
  p.vy = xadd(p.vy, xmul(ay, dt));
  p.vz = xadd(p.vz, xmul(0.0, dt));
  const double speed = xsqrt(xadd(xadd(xmul(p.vx, p.vx), xmul(p.vy, p.vy)), xmul(p.vz, p.vz)));
  if (p.coll == 'W') {
    const char w = p.wall;
    const bool sx = (w == 'x' || w == 'a' || w == 'b' || w == 'c');
    const bool sy = (w == 'y' || w == 'a' || w == 'b' || w == 'd');
    const bool sz = (w == 'z' || w == 'a' || w == 'c' || w == 'd');
    if (sx) p.px = p.px < 0.0 ? -xmul(P.Lx, 0.5) : xmul(P.Lx, 0.5);
    if (sy) p.py = p.py < 0.0 ? -xmul(P.Ly, 0.5) : xmul(P.Ly, 0.5);
    if (sz) p.pz = p.pz < 0.0 ? -xmul(P.Lz, 0.5) : xmul(P.Lz, 0.5);
    bool diffuse = false;
    if (P.diffuse > (double)FLT_MIN) diffuse = rng_uniform(p.rng) < P.diffuse;
    if (diffuse) {
      // cosine-law diffuse reflection (src/particle.cpp:309-328): both draws
      // now, the trigonometry now or (DEFER) batched later
      const double su = xsqrt(rng_uniform(p.rng));
      const double theta = xmul(xmul(rng_uniform(p.rng), 2.0), 3.141592653589793);
      if (w == 'x' || w == 'y' || w == 'z') {
        if (DEFER) {
          dd->x[0] = su;
          dd->x[1] = theta;
          dd->x[2] = speed;
          dd->wall = w;
          dd->gas = false;
          dd->pending = true;
        } else {
          diffuse_velocity(p, su, theta, speed, w);
        }
      } else {
        p.stop = true;  // a diffuse hit on an edge or corner stops the particle
      }
    } else {
      if (sx) p.vx = -p.vx;
      if (sy) p.vy = -p.vy;
      if (sz) p.vz = -p.vz;
    }
  } else if (GAS && p.coll == 'G') {
    if (DEFER && dd->gas) {
      // the three normals' uniform draws now, in rng_normal's order: the first
      // normal is the cached spare or opens pair 0, whose spare is the second;
      // the third opens pair 1 (its spare stays cached) or is pair 0's spare
      dd->spare_first = p.rng.has;
      marsaglia_draw(p.rng, dd->x[1], dd->x[2], dd->x[3]);
      if (!dd->spare_first) marsaglia_draw(p.rng, dd->x[4], dd->x[5], dd->x[6]);
      p.rng.has = !dd->spare_first;
      dd->pending = true;
    } else if (P.dist == 'M') {
      p.vx = xmul(rng_normal(p.rng, 0.0, 1.0), P.sqrtKT_m);
      p.vy = xmul(rng_normal(p.rng, 0.0, 1.0), P.sqrtKT_m);
      p.vz = xmul(rng_normal(p.rng, 0.0, 1.0), P.sqrtKT_m);
    } else if (P.dist == 'C') {
      const double dx = rng_normal(p.rng, 0.0, 1.0);
      const double dy = rng_normal(p.rng, 0.0, 1.0);
      const double dz = rng_normal(p.rng, 0.0, 1.0);
      const double nrm = xsqrt(xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz)));
      p.vx = xdiv(xmul(dx, speed), nrm);
      p.vy = xdiv(xmul(dy, speed), nrm);
      p.vz = xdiv(xmul(dz, speed), nrm);
    }
  }
  // ---- sanity_check
  const double tol = 1.0e-15;
  if (fabs(p.px) > xadd(hLx, tol) || fabs(p.py) > xadd(hLy, tol) || fabs(p.pz) > xadd(hLz, tol)) {
    p.stop = true; p.fail = 1;  // out of bounds
  } else if (isinf(s0.t) || isinf(p.t)) {
    p.stop = true; p.fail = 2;  // infinite time
  } else if (isnan(s0.px) || isnan(s0.py) || isnan(s0.pz) || isnan(p.px) || isnan(p.py) || isnan(p.pz)) {
    p.stop = true; p.fail = 3;  // NaN position
  } else if (isnan(p.vx) || isnan(p.vy) || isnan(p.vz) || isnan(s0.vx) || isnan(s0.vy) || isnan(s0.vz)) {
    p.stop = true; p.fail = 4;  // NaN velocity
  }
  return finished;
}

// ------------------------------------------------------------ field model
// Integrator state of the current segment.  Omega(tau) = gamma*B at time
// t0 + tau is the quadratic o0 + tau*(o1 + tau*o2) (plus the pulse).
struct Seg {
  double o0x, o0y, o0z, o1x, o1y, o1z, o2x, o2y, o2z;
#if !ST_GRAD_IS_LINEAR
  double p0x, p0y, p0z, v0x, v0y, v0z;
#endif
  double gpa;          // gamma * pulse amplitude (0: no pulse)
  double t0, xf, x, h, posneg, facold;
  double kx, ky, kz;   // DOP853: derivative at (x, y) (FSAL); RK45: last stage-6 state
  double lastH, lnprev;
  double hu;           // step size of the last accepted attempt (read by the adjoint replay)
  unsigned int nstep;
  int turns;           // precession turns of the segment's accepted steps (count_turn)
  bool reject, last;
  bool acc;            // the last attempt was accepted
};

// Precession phase accumulation: the phase phi = atan2(Sz, Sy) about x jumps
// by 2 pi where the spin's (y, z) projection crosses the cut at phi = +-pi
// (Sy < 0, Sz changing sign).  An accepted step at rtol 1e-12 turns the spin
// by far less than pi, so a crossing is a sign change of Sz with Sy < 0 at
// both ends, counted +1 from phi near +pi to near -pi (phi increasing) and -1
// back; atan2(Sz, Sy) + 2 pi * turns is then continuous along the run.
__device__ __forceinline__ int count_turn(double y0, double z0, double y1, double z1) {
  if (!(y0 < 0.0 && y1 < 0.0)) return 0;
  const bool s0 = signbit(z0), s1 = signbit(z1);
  return (s0 == s1) ? 0 : (s1 ? 1 : -1);
}

// The per-set field constants (launch_prepare_sets): gamma * B0, the gradient
// tensor's columns through the st_grad hook, gamma * E / c^2 and the gravity
// terms of the segment polynomial.
__device__ inline void prepare_set(SetParams& P) {
  const double gm = P.gamma;
  const double g_ = P.gravity ? kGravity : 0.0;
  P.gB0[0] = gm * P.B0x; P.gB0[1] = gm * P.B0y; P.gB0[2] = gm * P.B0z;
  const Vec3 ex = {1.0, 0.0, 0.0}, ey = {0.0, 1.0, 0.0}, ez = {0.0, 0.0, 1.0};
  const Vec3 c0 = st_grad(ex, P), c1 = st_grad(ey, P), c2 = st_grad(ez, P);
  P.gGc[0][0] = gm * c0.x; P.gGc[0][1] = gm * c0.y; P.gGc[0][2] = gm * c0.z;
  P.gGc[1][0] = gm * c1.x; P.gGc[1][1] = gm * c1.y; P.gGc[1][2] = gm * c1.z;
  P.gGc[2][0] = gm * c2.x; P.gGc[2][1] = gm * c2.y; P.gGc[2][2] = gm * c2.z;
  P.gEc[0] = gm * P.inv_c2 * P.Ex; P.gEc[1] = gm * P.inv_c2 * P.Ey; P.gEc[2] = gm * P.inv_c2 * P.Ez;
  // d/dtau of v x E along the parabola: (g yhat) x E = g (Ez, 0, -Ex)
  P.o1g[0] = gm * P.inv_c2 * g_ * P.Ez; P.o1g[1] = 0.0; P.o1g[2] = -gm * P.inv_c2 * g_ * P.Ex;
#if ST_GRAD_IS_LINEAR
  P.o2c[0] = 0.5 * g_ * P.gGc[1][0]; P.o2c[1] = 0.5 * g_ * P.gGc[1][1]; P.o2c[2] = 0.5 * g_ * P.gGc[1][2];
#else
  P.o2c[0] = P.o2c[1] = P.o2c[2] = 0.0;  // the hook is evaluated at every stage instead
#endif
}

// Coefficients o0, o1 of the field polynomial of a segment starting at (p0, v0).
__device__ __forceinline__ void seg_field(const SetParams& P, double px, double py, double pz, double vx, double vy,
                                          double vz, double o0[3], double o1[3]) {
  const double* e = P.gEc;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    // v0 x gEc, component c
    const double cr = (c == 0) ? fma(vy, e[2], -vz * e[1]) : (c == 1) ? fma(vz, e[0], -vx * e[2]) : fma(vx, e[1], -vy * e[0]);
#if ST_GRAD_IS_LINEAR
    o0[c] = P.gB0[c] + fma(px, P.gGc[0][c], fma(py, P.gGc[1][c], fma(pz, P.gGc[2][c], cr)));
    o1[c] = fma(vx, P.gGc[0][c], fma(vy, P.gGc[1][c], fma(vz, P.gGc[2][c], P.o1g[c])));
#else
    o0[c] = P.gB0[c] + cr;
    o1[c] = P.o1g[c];
#endif
  }
}

// Fill the integrator's segment from its field coefficients and time span.
__device__ __forceinline__ void seg_begin(Seg& g, const SetParams& P, double t0, double t_end, const double o0[3],
                                          const double o1[3]) {
  g.o0x = o0[0]; g.o0y = o0[1]; g.o0z = o0[2];
  g.o1x = o1[0]; g.o1y = o1[1]; g.o1z = o1[2];
  g.o2x = P.o2c[0]; g.o2y = P.o2c[1]; g.o2z = P.o2c[2];
  g.gpa = P.gamma * P.a;
  g.t0 = t0;
  g.xf = t_end;
  g.x = t0;
  g.posneg = (t_end - t0 < 0.0) ? -1.0 : 1.0;
}

__device__ __forceinline__ void seg_setup(Seg& g, const SetParams& P, const SegStart& s0, double t_end) {
  double o0[3], o1[3];
  seg_field(P, s0.px, s0.py, s0.pz, s0.vx, s0.vy, s0.vz, o0, o1);
  seg_begin(g, P, s0.t, t_end, o0, o1);
#if !ST_GRAD_IS_LINEAR
  g.p0x = s0.px; g.p0y = s0.py; g.p0z = s0.pz;
  g.v0x = s0.vx; g.v0y = s0.vy; g.v0z = s0.vz;
#endif
}

// Omega = gamma * B at tau = t - t0.
__device__ __forceinline__ void omega_at(const Seg& g, const SetParams& P, double tau, double& Ox, double& Oy,
                                         double& Oz) {
  Ox = fma(fma(g.o2x, tau, g.o1x), tau, g.o0x);
  Oy = fma(fma(g.o2y, tau, g.o1y), tau, g.o0y);
  Oz = fma(fma(g.o2z, tau, g.o1z), tau, g.o0z);
#if !ST_GRAD_IS_LINEAR
  {
    const double gy = P.gravity ? 0.5 * kGravity : 0.0;
    const Vec3 pos = {fma(g.v0x, tau, g.p0x), fma(fma(gy, tau, g.v0y), tau, g.p0y), fma(g.v0z, tau, g.p0z)};
    const Vec3 Gp = st_grad(pos, P);
    Ox = fma(P.gamma, Gp.x, Ox);
    Oy = fma(P.gamma, Gp.y, Oy);
    Oz = fma(P.gamma, Gp.z, Oz);
  }
#endif
#if ST_PULSE_IS_Z_COS
  if (g.gpa != 0.0) Oz = fma(g.gpa, cos(P.w * (g.t0 + tau)), Oz);
#else
  {
    const Vec3 pu = st_pulse(g.t0 + tau, P);
    Ox = fma(P.gamma, pu.x, Ox);
    Oy = fma(P.gamma, pu.y, Oy);
    Oz = fma(P.gamma, pu.z, Oz);
  }
#endif
}

// Bloch right-hand side f = y x Omega (src/integrator.cpp:83-88).
__device__ __forceinline__ void bloch(double yx, double yy, double yz, double Ox, double Oy, double Oz, double& fx,
                                      double& fy, double& fz) {
  fx = fma(yy, Oz, -yz * Oy);
  fy = fma(yz, Ox, -yx * Oz);
  fz = fma(yx, Oy, -yy * Ox);
}

__device__ __forceinline__ void feval(const Seg& g, const SetParams& P, double tau, double yx, double yy, double yz,
                                      double& fx, double& fy, double& fz) {
  double Ox, Oy, Oz;
  omega_at(g, P, tau, Ox, Oy, Oz);
  bloch(yx, yy, yz, Ox, Oy, Oz, fx, fy, fz);
}

// The field polynomial scaled by a step size h, so that a stage's Bloch
// evaluation gives h k directly and its state y + sum a_j (h k_j) is an FMA
// chain from y (ten multiplications per attempt instead of one per stage and
// component).
struct HPoly {
  double o0x, o0y, o0z, o1x, o1y, o1z, o2x, o2y, o2z, gpa, h;
};
__device__ __forceinline__ HPoly hpoly_of(const Seg& g, double h) {
  return {h * g.o0x, h * g.o0y, h * g.o0z, h * g.o1x, h * g.o1y, h * g.o1z,
          h * g.o2x, h * g.o2y, h * g.o2z, h * g.gpa, h};
}
// h Omega at tau = t - t0 (omega_at, scaled).
__device__ __forceinline__ void homega_at(const HPoly& q, const Seg& g, const SetParams& P, double tau, double& Ox,
                                          double& Oy, double& Oz) {
  Ox = fma(fma(q.o2x, tau, q.o1x), tau, q.o0x);
  Oy = fma(fma(q.o2y, tau, q.o1y), tau, q.o0y);
  Oz = fma(fma(q.o2z, tau, q.o1z), tau, q.o0z);
#if !ST_GRAD_IS_LINEAR
  {
    const double gy = P.gravity ? 0.5 * kGravity : 0.0;
    const Vec3 pos = {fma(g.v0x, tau, g.p0x), fma(fma(gy, tau, g.v0y), tau, g.p0y), fma(g.v0z, tau, g.p0z)};
    const Vec3 Gp = st_grad(pos, P);
    const double hg = q.h * P.gamma;
    Ox = fma(hg, Gp.x, Ox);
    Oy = fma(hg, Gp.y, Oy);
    Oz = fma(hg, Gp.z, Oz);
  }
#endif
#if ST_PULSE_IS_Z_COS
  if (g.gpa != 0.0) Oz = fma(q.gpa, cos(P.w * (g.t0 + tau)), Oz);
#else
  {
    const Vec3 pu = st_pulse(g.t0 + tau, P);
    const double hg = q.h * P.gamma;
    Ox = fma(hg, pu.x, Ox);
    Oy = fma(hg, pu.y, Oy);
    Oz = fma(hg, pu.z, Oz);
  }
#endif
}

// ------------------------------------------------------------ DOP853
// Start a DOP853 call over the segment (src/integrator.cpp:102-119).
__device__ __forceinline__ void dop_begin(Seg& g, const SetParams& P, double Sx, double Sy, double Sz, double h) {
  g.h = h;
  g.facold = 1.0e-4;
  g.nstep = 0;
  g.turns = 0;
  g.reject = false;
  g.last = false;
  feval(g, P, 0.0, Sx, Sy, Sz, g.kx, g.ky, g.kz);
}

// DOP853 stage structure as constexpr functions of compile-time stage and
// term indices (they fold to constants inside unrolled loops).
namespace dopst {
// earlier stages summed into stage s (2..12): stage 1, then 2 (s = 3),
// 3.. (s = 4, 5) or 4.. (s >= 6)
__device__ __forceinline__ constexpr int src(int s, int j) { return j == 0 ? 1 : (s == 3 ? 2 : (s <= 5 ? j + 2 : j + 3)); }
__device__ __forceinline__ constexpr int cnt(int s) { return s <= 2 ? s - 1 : (s <= 4 ? 2 : (s == 5 ? 3 : s - 3)); }
// coefficient of term j of stage s (the a_{s,src(s,j)} of the tableau)
__device__ __forceinline__ constexpr double a(int s, int j) {
  switch (s * 16 + j) {
    case 32: return dop::A21;
    case 48: return dop::A31;
    case 49: return dop::A32;
    case 64: return dop::A41;
    case 65: return dop::A43;
    case 80: return dop::A51;
    case 81: return dop::A53;
    case 82: return dop::A54;
    case 96: return dop::A61;
    case 97: return dop::A64;
    case 98: return dop::A65;
    case 112: return dop::A71;
    case 113: return dop::A74;
    case 114: return dop::A75;
    case 115: return dop::A76;
    case 128: return dop::A81;
    case 129: return dop::A84;
    case 130: return dop::A85;
    case 131: return dop::A86;
    case 132: return dop::A87;
    case 144: return dop::A91;
    case 145: return dop::A94;
    case 146: return dop::A95;
    case 147: return dop::A96;
    case 148: return dop::A97;
    case 149: return dop::A98;
    case 160: return dop::A101;
    case 161: return dop::A104;
    case 162: return dop::A105;
    case 163: return dop::A106;
    case 164: return dop::A107;
    case 165: return dop::A108;
    case 166: return dop::A109;
    case 176: return dop::A111;
    case 177: return dop::A114;
    case 178: return dop::A115;
    case 179: return dop::A116;
    case 180: return dop::A117;
    case 181: return dop::A118;
    case 182: return dop::A119;
    case 183: return dop::A1110;
    case 192: return dop::A121;
    case 193: return dop::A124;
    case 194: return dop::A125;
    case 195: return dop::A126;
    case 196: return dop::A127;
    case 197: return dop::A128;
    case 198: return dop::A129;
    case 199: return dop::A1210;
    case 200: return dop::A1211;
    default: return 0.0;
  }
}
// node of stage s (stage 12 at x + h)
__device__ __forceinline__ constexpr double c(int s) {
  switch (s) {
    case 2: return dop::C2;
    case 3: return dop::C3;
    case 4: return dop::C4;
    case 5: return dop::C5;
    case 6: return dop::C6;
    case 7: return dop::C7;
    case 8: return dop::C8;
    case 9: return dop::C9;
    case 10: return dop::C10;
    case 11: return dop::C11;
    case 12: return 1.0;
    default: return 0.0;
  }
}
// 8th-order weight of stage s
__device__ __forceinline__ constexpr double b(int s) {
  switch (s) {
    case 1: return dop::B1;
    case 6: return dop::B6;
    case 7: return dop::B7;
    case 8: return dop::B8;
    case 9: return dop::B9;
    case 10: return dop::B10;
    case 11: return dop::B11;
    case 12: return dop::B12;
    default: return 0.0;
  }
}
}  // namespace dopst

// Where an attempt keeps its stage derivatives k2..k11 (k1 and k12 stay in
// registers): registers (a local array that the unrolled code indexes with
// constants), or this thread's column of a [10][3][BLOCK] shared-memory
// array, which frees ~30 registers per thread.
struct StageRegs {
  double v[12][3];
  __device__ __forceinline__ double& k(int s, int c) { return v[s][c]; }
};
struct StageSmem {
  double* base;  // &array[0][0][thread]
  int stride;    // BLOCK
  __device__ __forceinline__ double& k(int s, int c) { return base[((s - 2) * 3 + c) * stride]; }
};

// One attempted DOP853 step (one pass of the loop at src/integrator.cpp:128-247),
// stage derivatives in `ks`.  Returns 0 to continue, 1 when the segment's last
// step was accepted (g.h then holds that step, as the reference returns it),
// -1 after more than nmax attempts.
template <class KS>
__device__ __forceinline__ int dop_attempt_ks(Seg& g, const SetParams& P, double& Sx, double& Sy, double& Sz,
                                              KS& ks) {
  using namespace dop;
  if (g.nstep > P.nmax) return -1;
  double h = g.h;
  bool last = g.last;
  if ((g.x + 1.01 * h - g.xf) * g.posneg > 0.0) {
    h = g.xf - g.x;
    last = true;
  }
  if (h < P.hmin && !last) h = P.hmin;
  g.nstep++;
  g.acc = false;
  const double tx = g.x - g.t0;
  const double S0[3] = {Sx, Sy, Sz};
  // stage derivatives are carried scaled by h (ks holds h k_s)
  const HPoly hp = hpoly_of(g, h);
  const double k1[3] = {h * g.kx, h * g.ky, h * g.kz};
  // stages 2..11: y + sum_j a_sj (h k_j), then h k_s = Y x (h Omega(x + c_s h))
#pragma unroll
  for (int s = 2; s <= 11; ++s) {
    double Y[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double acc = fma(dopst::a(s, 0), k1[c], S0[c]);
#pragma unroll
      for (int j = 1; j < dopst::cnt(s); ++j) acc = fma(dopst::a(s, j), ks.k(dopst::src(s, j), c), acc);
      Y[c] = acc;
    }
    double Ox, Oy, Oz, kx, ky, kz;
    homega_at(hp, g, P, fma(dopst::c(s), h, tx), Ox, Oy, Oz);
    bloch(Y[0], Y[1], Y[2], Ox, Oy, Oz, kx, ky, kz);
    ks.k(s, 0) = kx;
    ks.k(s, 1) = ky;
    ks.k(s, 2) = kz;
  }
  // stage 12 at x + h; its unscaled Omega is reused for the FSAL derivative
  double Y12[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double acc = fma(dopst::a(12, 0), k1[c], S0[c]);
#pragma unroll
    for (int j = 1; j < dopst::cnt(12); ++j) acc = fma(dopst::a(12, j), ks.k(dopst::src(12, j), c), acc);
    Y12[c] = acc;
  }
  const double tph = tx + h;
  double Ox12, Oy12, Oz12, k12[3];
  omega_at(g, P, tph, Ox12, Oy12, Oz12);
  bloch(Y12[0], Y12[1], Y12[2], h * Ox12, h * Oy12, h * Oz12, k12[0], k12[1], k12[2]);
  // 8th-order combination and the new state
  double bsum[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double acc = B1 * k1[c];
    acc = fma(B6, ks.k(6, c), acc);
    acc = fma(B7, ks.k(7, c), acc);
    acc = fma(B8, ks.k(8, c), acc);
    acc = fma(B9, ks.k(9, c), acc);
    acc = fma(B10, ks.k(10, c), acc);
    acc = fma(B11, ks.k(11, c), acc);
    bsum[c] = fma(B12, k12[c], acc);
  }
  const double bx = bsum[0], by = bsum[1], bz = bsum[2];
  const double nx = Sx + bx, ny = Sy + by, nz = Sz + bz;
  // error estimates: 3rd-order (bhh) and 5th-order (er) rows, h times the
  // reference's; the scale cancels in err = |h| err_5 / sqrt(3 (err_5 + 0.01 err_3))
  const double e1x = fma(-BHH3, k12[0], fma(-BHH2, ks.k(9, 0), fma(-BHH1, k1[0], bx)));
  const double e1y = fma(-BHH3, k12[1], fma(-BHH2, ks.k(9, 1), fma(-BHH1, k1[1], by)));
  const double e1z = fma(-BHH3, k12[2], fma(-BHH2, ks.k(9, 2), fma(-BHH1, k1[2], bz)));
  double er[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    double acc = ER1 * k1[c];
    acc = fma(ER6, ks.k(6, c), acc);
    acc = fma(ER7, ks.k(7, c), acc);
    acc = fma(ER8, ks.k(8, c), acc);
    acc = fma(ER9, ks.k(9, c), acc);
    acc = fma(ER10, ks.k(10, c), acc);
    acc = fma(ER11, ks.k(11, c), acc);
    er[c] = fma(ER12, k12[c], acc);
  }
  const double ax = er[0], ay = er[1], az = er[2];
  const double wx = rcp_full(fma(P.rtol, max_d(fabs(Sx), fabs(nx)), P.atol));
  const double wy = rcp_full(fma(P.rtol, max_d(fabs(Sy), fabs(ny)), P.atol));
  const double wz = rcp_full(fma(P.rtol, max_d(fabs(Sz), fabs(nz)), P.atol));
  const double q1x = e1x * wx, q1y = e1y * wy, q1z = e1z * wz;
  const double q2x = ax * wx, q2y = ay * wy, q2z = az * wz;
  const double err2 = fma(q1z, q1z, fma(q1y, q1y, q1x * q1x));
  double err = fma(q2z, q2z, fma(q2y, q2y, q2x * q2x));
  double deno = fma(0.01, err2, err);
  if (deno <= 0.0) deno = 1.0;
  err = err * rsqrt_full(deno * 3.0);
  // step-size controller (Lund-stabilised, clamped to [1/fac2, 1/fac1])
  double hnew;
  const bool fast = (P.beta == 0.0) && (err > 1e-300) && (err < 1e300);
  double rr = 0.0, fac11 = 0.0;
  if (fast) {
    rr = rroot8(err);  // 1 / fac11
    hnew = h * min_d(P.fac2, max_d(P.fac1, P.safe * rr));
  } else {
    fac11 = pow(err, P.expo1);
    double fac = fac11 / pow(g.facold, P.beta);
    fac = max_d(P.facc2, min_d(P.facc1, fac / P.safe));
    hnew = h / fac;
  }
  int ret = 0;
  if (err <= 1.0 || P.fixed) {
    g.acc = true;
    g.hu = h;
    g.facold = max_d(err, 1.0e-4);
    bloch(nx, ny, nz, Ox12, Oy12, Oz12, g.kx, g.ky, g.kz);  // FSAL: f(x + h, y_new)
    g.turns += count_turn(Sy, Sz, ny, nz);
    Sx = nx; Sy = ny; Sz = nz;
    g.x = g.x + h;
    if (last) {
      g.h = h;
      g.last = true;
      return 1;
    }
    if (fabs(hnew) > P.hmax) hnew = g.posneg * P.hmax;
    if (g.reject) hnew = g.posneg * min_d(fabs(hnew), fabs(h));
    g.reject = false;
  } else {
    hnew = fast ? h * max_d(P.fac1, P.safe * rr) : h / min_d(P.facc1, fac11 / P.safe);
    g.reject = true;
    last = false;
  }
  g.last = last;
  g.h = P.fixed ? h : hnew;
  return ret;
}


// One attempted DOP853 step with the stage derivatives in registers.
__device__ __forceinline__ int dop_attempt(Seg& g, const SetParams& P, double& Sx, double& Sy, double& Sz) {
  StageRegs ks;
  return dop_attempt_ks(g, P, Sx, Sy, Sz, ks);
}

// ------------------------------------------------------------ RK45
__device__ __forceinline__ void rk45_begin(Seg& g, double h) {
  g.h = h;
  g.lastH = h;
  g.lnprev = 0.0;  // log(prev_ratio = 1)
  g.kx = g.ky = g.kz = 0.0;  // the stage state a fresh call starts from
  g.nstep = 0;
  g.turns = 0;
  g.last = false;
}

// One attempt of integrateRK45 (src/integrator.cpp:267-335), including its
// first-stage quirk: k1 is evaluated at the previous attempt's last stage
// state (zero on the first attempt of a call).  Returns 0 to continue, 1 when
// the segment end was reached (g.h then holds the carried step), -1 when
// h < hmin, -2 after more than nmax attempts.
__device__ __forceinline__ int rk45_attempt(Seg& g, const SetParams& P, double& Sx, double& Sy, double& Sz) {
  using namespace rk45;
  g.nstep++;
  if (g.nstep > P.nmax) return -2;
  const double endDt = g.xf - g.x;
  double h = g.h;
  g.lastH = h;
  if (P.fixed) {
    h = P.h0;
  } else {
    if (h > P.hmax)
      h = std_min(h, P.hmax);
    else if (h < P.hmin)
      return -1;
  }
  bool stop;
  if (h >= endDt) {
    h = endDt;
    stop = true;
  } else {
    g.lastH = h;
    stop = false;
  }
  const double tx = g.x - g.t0;
  // stage derivatives scaled by h (k below is h f), as in the DOP853 attempt
  const HPoly hp = hpoly_of(g, h);
  double k1x, k1y, k1z, k2x, k2y, k2z, k3x, k3y, k3z, k4x, k4y, k4z, k5x, k5y, k5z, k6x, k6y, k6z;
  double yx, yy, yz, Ox, Oy, Oz;
  homega_at(hp, g, P, tx, Ox, Oy, Oz);
  bloch(g.kx, g.ky, g.kz, Ox, Oy, Oz, k1x, k1y, k1z);
  yx = fma(B21, k1x, Sx); yy = fma(B21, k1y, Sy); yz = fma(B21, k1z, Sz);
  homega_at(hp, g, P, fma(A2, h, tx), Ox, Oy, Oz);
  bloch(yx, yy, yz, Ox, Oy, Oz, k2x, k2y, k2z);
  yx = fma(B32, k2x, fma(B31, k1x, Sx));
  yy = fma(B32, k2y, fma(B31, k1y, Sy));
  yz = fma(B32, k2z, fma(B31, k1z, Sz));
  homega_at(hp, g, P, fma(A3, h, tx), Ox, Oy, Oz);
  bloch(yx, yy, yz, Ox, Oy, Oz, k3x, k3y, k3z);
  yx = fma(B43, k3x, fma(B42, k2x, fma(B41, k1x, Sx)));
  yy = fma(B43, k3y, fma(B42, k2y, fma(B41, k1y, Sy)));
  yz = fma(B43, k3z, fma(B42, k2z, fma(B41, k1z, Sz)));
  homega_at(hp, g, P, fma(A4, h, tx), Ox, Oy, Oz);
  bloch(yx, yy, yz, Ox, Oy, Oz, k4x, k4y, k4z);
  yx = fma(B54, k4x, fma(B53, k3x, fma(B52, k2x, fma(B51, k1x, Sx))));
  yy = fma(B54, k4y, fma(B53, k3y, fma(B52, k2y, fma(B51, k1y, Sy))));
  yz = fma(B54, k4z, fma(B53, k3z, fma(B52, k2z, fma(B51, k1z, Sz))));
  homega_at(hp, g, P, fma(A5, h, tx), Ox, Oy, Oz);
  bloch(yx, yy, yz, Ox, Oy, Oz, k5x, k5y, k5z);
  yx = fma(B65, k5x, fma(B64, k4x, fma(B63, k3x, fma(B62, k2x, fma(B61, k1x, Sx)))));
  yy = fma(B65, k5y, fma(B64, k4y, fma(B63, k3y, fma(B62, k2y, fma(B61, k1y, Sy)))));
  yz = fma(B65, k5z, fma(B64, k4z, fma(B63, k3z, fma(B62, k2z, fma(B61, k1z, Sz)))));
  homega_at(hp, g, P, fma(A6, h, tx), Ox, Oy, Oz);
  bloch(yx, yy, yz, Ox, Oy, Oz, k6x, k6y, k6z);
  g.kx = yx; g.ky = yy; g.kz = yz;  // the next attempt's first stage sees this state
  // CH2 and CT2 are zero: k2 does not enter the weights; the new state adds
  // the small weighted sum to S in one rounding
  const double wx = fma(CH6, k6x, fma(CH5, k5x, fma(CH4, k4x, fma(CH3, k3x, CH1 * k1x))));
  const double wy = fma(CH6, k6y, fma(CH5, k5y, fma(CH4, k4y, fma(CH3, k3y, CH1 * k1y))));
  const double wz = fma(CH6, k6z, fma(CH5, k5z, fma(CH4, k4z, fma(CH3, k3z, CH1 * k1z))));
  const double tex = fma(CT6, k6x, fma(CT5, k5x, fma(CT4, k4x, fma(CT3, k3x, CT1 * k1x))));
  const double tey = fma(CT6, k6y, fma(CT5, k5y, fma(CT4, k4y, fma(CT3, k3y, CT1 * k1y))));
  const double tez = fma(CT6, k6z, fma(CT5, k5z, fma(CT4, k4z, fma(CT3, k3z, CT1 * k1z))));
  double error = sqrt(fma(tez, tez, fma(tey, tey, tex * tex)));
  error = std_max(error, 1.0e-16);
  const double ratio = P.rtol / error;
  const double lnr = log(ratio);
  double q = exp(E1 * lnr + E2 * g.lnprev);  // ratio^E1 * prev_ratio^E2
  q = std_min(q, 4.0);
  if ((q > 0.81 && error < 2.0 * P.rtol) || P.fixed) {
    const double ny = Sy + wy, nz = Sz + wz;
    g.turns += count_turn(Sy, Sz, ny, nz);
    Sx = Sx + wx; Sy = ny; Sz = nz;
    g.x += h;
    if (stop) {
      g.h = g.lastH;
      return 1;
    }
  }
  g.h = P.fixed ? h : h * q;
  g.lnprev = lnr;
  return 0;
}

// ------------------------------------------------------------ integrator types 2-5
// Magnus CFET8 (src/integrator.cpp:625-722), RK45 with quaternions (:441-528),
// RKF45 (:339-439) and RKF45 with quaternions (:530-623).
namespace cfetc {
__device__ __forceinline__ constexpr double x(int i) {
  return i == 0 ? cfet::X1 : i == 1 ? cfet::X2 : i == 2 ? cfet::X3 : i == 3 ? cfet::X4 : cfet::X5;
}
// CFET8 row r (0-5), node j (0-4)
__device__ __forceinline__ constexpr double g(int r, int j) {
  switch (r * 8 + j) {
    case 0: return cfet::G11;  case 1: return cfet::G12;  case 2: return cfet::G13;
    case 3: return cfet::G14;  case 4: return cfet::G15;
    case 8: return cfet::G21;  case 9: return cfet::G22;  case 10: return cfet::G23;
    case 11: return cfet::G24; case 12: return cfet::G25;
    case 16: return cfet::G31; case 17: return cfet::G32; case 18: return cfet::G33;
    case 19: return cfet::G34; case 20: return cfet::G35;
    case 24: return cfet::G41; case 25: return cfet::G42; case 26: return cfet::G43;
    case 27: return cfet::G44; case 28: return cfet::G45;
    case 32: return cfet::G51; case 33: return cfet::G52; case 34: return cfet::G53;
    case 35: return cfet::G54; case 36: return cfet::G55;
    case 40: return cfet::G61; case 41: return cfet::G62; case 42: return cfet::G63;
    case 43: return cfet::G64; default: return cfet::G65;
  }
}
// CFET6 row r (0-2), node j (0-4)
__device__ __forceinline__ constexpr double hh(int r, int j) {
  switch (r * 8 + j) {
    case 0: return cfet::H11;  case 1: return cfet::H12;  case 2: return cfet::H13;
    case 3: return cfet::H14;  case 4: return cfet::H15;
    case 8: return cfet::H21;  case 9: return cfet::H22;  case 10: return cfet::H23;
    case 11: return cfet::H24; case 12: return cfet::H25;
    case 16: return cfet::H31; case 17: return cfet::H32; case 18: return cfet::H33;
    case 19: return cfet::H34; default: return cfet::H35;
  }
}
}  // namespace cfetc

// v rotated by the angle |k| about -k/|k|: Rodrigues' formula
// v cos + (v x k) sin/|k| + k (k.v)(1 - cos)/|k|^2 (rodriguez, src/quaternion.cpp).
// One reciprocal square root gives |k|, 1/|k| and 1/|k|^2 (the reference
// takes a square root and two divisions).
__device__ __forceinline__ void rodrigues(double kx, double ky, double kz, double& vx, double& vy, double& vz) {
  const double a2 = fma(kz, kz, fma(ky, ky, kx * kx));
  const double r = rsqrt(a2);
  const double angle = a2 * r;
  double s, c;
  sincos(angle, &s, &c);
  const double sa = s * r;
  const double d = fma(kz, vz, fma(ky, vy, kx * vx)) * (1.0 - c) * (r * r);
  const double cx = fma(vy, kz, -vz * ky), cy = fma(vz, kx, -vx * kz), cz = fma(vx, ky, -vy * kx);
  vx = fma(kx, d, fma(cx, sa, vx * c));
  vy = fma(ky, d, fma(cy, sa, vy * c));
  vz = fma(kz, d, fma(cz, sa, vz * c));
}

struct Quat {
  double w, x, y, z;
};

// Rotation by the angle |k| dt about -k/|k| as a unit quaternion
// (rodriguezQuat, src/quaternion.cpp).
__device__ __forceinline__ Quat rot_quat(double kx, double ky, double kz, double dt) {
  const double a2 = fma(kz, kz, fma(ky, ky, kx * kx));
  const double r = rsqrt(a2);
  double s, c;
  sincos(a2 * r * dt * 0.5, &s, &c);
  const double f = -s * r;
  return {c, kx * f, ky * f, kz * f};
}

// a b (qMult, src/quaternion.cpp)
__device__ __forceinline__ Quat qmul(const Quat& a, const Quat& b) {
  return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
          a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z, a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x};
}

// q (0, v) q* (qv_mult, src/quaternion.cpp), the terms of the pure
// quaternion's zero real part left out.
__device__ __forceinline__ void qrotate(const Quat& q, double vx, double vy, double vz, double& ox, double& oy,
                                        double& oz) {
  const double tw = -(q.x * vx + q.y * vy + q.z * vz);
  const double tx = q.w * vx + q.y * vz - q.z * vy;
  const double ty = q.w * vy + q.z * vx - q.x * vz;
  const double tz = q.w * vz + q.x * vy - q.y * vx;
  // (tw, tx, ty, tz) (q.w, -q.x, -q.y, -q.z)
  ox = -tw * q.x + tx * q.w - ty * q.z + tz * q.y;
  oy = -tw * q.y + ty * q.w - tz * q.x + tx * q.z;
  oz = -tw * q.z + tz * q.w - tx * q.y + ty * q.x;
}

// The Magnus stepper's 16 exponents in the order they are applied: the
// CFET8 exponents 11 down to 1 (rows 1..5 with the node order reversed, then
// rows 6..1), then the CFET6 exponents 5 down to 1 (rows 1, 2 reversed, then
// rows 3..1); entry [n][j] weights the field at node j.  The stepper reads
// them in a rolled loop, so the rotation code (with its sincos) appears once
// in the kernel instead of 16 times: the unrolled form stalled on
// instruction fetch.
constexpr int magnus_row(int n) { return n < 5 ? n : (n < 11 ? 10 - n : (n < 13 ? n - 11 : 15 - n)); }
constexpr bool magnus_rev(int n) { return n < 5 || n == 11 || n == 12; }
#define ST_MAGNUS_ROW(n)                                                                                      \
  {n < 11 ? cfetc::g(magnus_row(n), magnus_rev(n) ? 4 : 0) : cfetc::hh(magnus_row(n), magnus_rev(n) ? 4 : 0), \
   n < 11 ? cfetc::g(magnus_row(n), magnus_rev(n) ? 3 : 1) : cfetc::hh(magnus_row(n), magnus_rev(n) ? 3 : 1), \
   n < 11 ? cfetc::g(magnus_row(n), 2) : cfetc::hh(magnus_row(n), 2),                                        \
   n < 11 ? cfetc::g(magnus_row(n), magnus_rev(n) ? 1 : 3) : cfetc::hh(magnus_row(n), magnus_rev(n) ? 1 : 3), \
   n < 11 ? cfetc::g(magnus_row(n), magnus_rev(n) ? 0 : 4) : cfetc::hh(magnus_row(n), magnus_rev(n) ? 0 : 4)}
static __constant__ double kMagnusExp[16][5] = {
    ST_MAGNUS_ROW(0),  ST_MAGNUS_ROW(1),  ST_MAGNUS_ROW(2),  ST_MAGNUS_ROW(3),  ST_MAGNUS_ROW(4),  ST_MAGNUS_ROW(5),
    ST_MAGNUS_ROW(6),  ST_MAGNUS_ROW(7),  ST_MAGNUS_ROW(8),  ST_MAGNUS_ROW(9),  ST_MAGNUS_ROW(10), ST_MAGNUS_ROW(11),
    ST_MAGNUS_ROW(12), ST_MAGNUS_ROW(13), ST_MAGNUS_ROW(14), ST_MAGNUS_ROW(15)};
#undef ST_MAGNUS_ROW

// Magnus: the CFET8 product (exponents 11 down to 1, each a combination of h
// times the field at the five Gauss-Legendre nodes) gives the proposal, the
// CFET6 product beside it the error vector.
__device__ __forceinline__ void magnus_stages(const Seg& g, const SetParams& P, double tx, double h, double Sx,
                                              double Sy, double Sz, double w[3], double e[3]) {
  double B[5][3];  // h Omega at the nodes: the exponents are combinations of these
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    omega_at(g, P, fma(cfetc::x(i), h, tx), B[i][0], B[i][1], B[i][2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) B[i][c] *= h;
  }
  double y[3] = {Sx, Sy, Sz}, y8[3];
#pragma unroll 1
  for (int n = 0; n < 16; ++n) {
    if (n == 11) {  // CFET8 done: start CFET6 from S
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        y8[c] = y[c];
        y[c] = c == 0 ? Sx : (c == 1 ? Sy : Sz);
      }
    }
    const double* cf = kMagnusExp[n];
    double k[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double s = cf[0] * B[0][c];
#pragma unroll
      for (int j = 1; j < 5; ++j) s = fma(cf[j], B[j][c], s);
      k[c] = s;
    }
    rodrigues(k[0], k[1], k[2], y[0], y[1], y[2]);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    w[c] = y8[c];
    e[c] = y8[c] - y[c];
  }
}

// Per stage m (stages 1, 3, 4, 5, 6; stage 2's weights are zero): node,
// weight of the proposal's rotation, weight of the comparison's (RK45 only).
static __constant__ double kQuatStages[2][5][3] = {
    {{0.0, rk45::CH1, rk45::C1}, {rk45::A3, rk45::CH3, rk45::C3}, {rk45::A4, rk45::CH4, rk45::C4},
     {rk45::A5, rk45::CH5, rk45::C5}, {rk45::A6, rk45::CH6, 0.0}},
    {{0.0, rkf45::C1, 0.0}, {rkf45::A3, rkf45::C3, 0.0}, {rkf45::A4, rkf45::C4, 0.0}, {rkf45::A5, rkf45::C5, 0.0},
     {rkf45::A6, rkf45::C6, 0.0}}};

// RK45 / RKF45 with quaternions: the field at the stages' nodes, each turned
// into a rotation by h times a weight and composed (the first factor onto the
// identity, which is exact); the proposal uses the higher-order weights
// (RK45: CH1..CH6, RKF45: C1..C6), the comparison rotation the first five
// lower-order ones (RK45: C1..C5; RKF45: its own C1..C5, so the two products
// share all but the last factor).  A rolled loop keeps one copy of the
// rotation code in the kernel.
template <bool F>
__device__ __forceinline__ void quat_stages(const Seg& g, const SetParams& P, double tx, double h, double Sx,
                                            double Sy, double Sz, double w[3], double e[3]) {
  Quat qw = {1.0, 0.0, 0.0, 0.0}, qe = {1.0, 0.0, 0.0, 0.0};
#pragma unroll 1
  for (int m = 0; m < 5; ++m) {
    const double* cf = kQuatStages[F ? 1 : 0][m];
    double Ox, Oy, Oz;
    omega_at(g, P, fma(cf[0], h, tx), Ox, Oy, Oz);
    if (F) {
      const Quat r = rot_quat(Ox, Oy, Oz, h * cf[1]);
      if (m < 4)
        qe = qmul(r, qe);
      else
        qw = qmul(r, qe);
    } else {
      qw = qmul(rot_quat(Ox, Oy, Oz, h * cf[1]), qw);
      if (m < 4) qe = qmul(rot_quat(Ox, Oy, Oz, h * cf[2]), qe);
    }
  }
  double cx, cy, cz;
  qrotate(qw, Sx, Sy, Sz, w[0], w[1], w[2]);
  qrotate(qe, Sx, Sy, Sz, cx, cy, cz);
  e[0] = w[0] - cx;
  e[1] = w[1] - cy;
  e[2] = w[2] - cz;
}

// RKF45 with RK45's first-stage quirk (k1 at the previous attempt's last
// stage state, kept in g.k); its error vector is h times the whole
// fourth-order combination, as the reference computes it.
__device__ __forceinline__ void rkf45_stages(Seg& g, const SetParams& P, double tx, double h, double Sx, double Sy,
                                             double Sz, double w[3], double e[3]) {
  using namespace rkf45;
  double k1x, k1y, k1z, k2x, k2y, k2z, k3x, k3y, k3z, k4x, k4y, k4z, k5x, k5y, k5z, k6x, k6y, k6z;
  double yx, yy, yz;
  feval(g, P, tx, g.kx, g.ky, g.kz, k1x, k1y, k1z);
  yx = fma(h * B21, k1x, Sx); yy = fma(h * B21, k1y, Sy); yz = fma(h * B21, k1z, Sz);
  feval(g, P, fma(A2, h, tx), yx, yy, yz, k2x, k2y, k2z);
  yx = fma(h, fma(B32, k2x, B31 * k1x), Sx);
  yy = fma(h, fma(B32, k2y, B31 * k1y), Sy);
  yz = fma(h, fma(B32, k2z, B31 * k1z), Sz);
  feval(g, P, fma(A3, h, tx), yx, yy, yz, k3x, k3y, k3z);
  yx = fma(h, fma(B43, k3x, fma(B42, k2x, B41 * k1x)), Sx);
  yy = fma(h, fma(B43, k3y, fma(B42, k2y, B41 * k1y)), Sy);
  yz = fma(h, fma(B43, k3z, fma(B42, k2z, B41 * k1z)), Sz);
  feval(g, P, fma(A4, h, tx), yx, yy, yz, k4x, k4y, k4z);
  yx = fma(h, fma(B54, k4x, fma(B53, k3x, fma(B52, k2x, B51 * k1x))), Sx);
  yy = fma(h, fma(B54, k4y, fma(B53, k3y, fma(B52, k2y, B51 * k1y))), Sy);
  yz = fma(h, fma(B54, k4z, fma(B53, k3z, fma(B52, k2z, B51 * k1z))), Sz);
  feval(g, P, fma(A5, h, tx), yx, yy, yz, k5x, k5y, k5z);
  yx = fma(h, fma(B65, k5x, fma(B64, k4x, fma(B63, k3x, fma(B62, k2x, B61 * k1x)))), Sx);
  yy = fma(h, fma(B65, k5y, fma(B64, k4y, fma(B63, k3y, fma(B62, k2y, B61 * k1y)))), Sy);
  yz = fma(h, fma(B65, k5z, fma(B64, k4z, fma(B63, k3z, fma(B62, k2z, B61 * k1z)))), Sz);
  feval(g, P, fma(A6, h, tx), yx, yy, yz, k6x, k6y, k6z);
  g.kx = yx; g.ky = yy; g.kz = yz;
  w[0] = fma(h, fma(C6, k6x, fma(C5, k5x, fma(C4, k4x, fma(C3, k3x, C1 * k1x)))), Sx);
  w[1] = fma(h, fma(C6, k6y, fma(C5, k5y, fma(C4, k4y, fma(C3, k3y, C1 * k1y)))), Sy);
  w[2] = fma(h, fma(C6, k6z, fma(C5, k5z, fma(C4, k4z, fma(C3, k3z, C1 * k1z)))), Sz);
  e[0] = h * fma(CR5, k5x, fma(CR4, k4x, fma(CR3, k3x, CR1 * k1x)));
  e[1] = h * fma(CR5, k5y, fma(CR4, k4y, fma(CR3, k3y, CR1 * k1y)));
  e[2] = h * fma(CR5, k5z, fma(CR4, k4z, fma(CR3, k3z, CR1 * k1z)));
}

// Start a type 2-5 call over the segment: the same state as RK45's.
__device__ __forceinline__ void ext_begin(Seg& g, double h) { rk45_begin(g, h); }

// One attempt of integrator type 2-5 (P.integrator).  Their shared step
// controller differs from RK45's: the segment end is tested before the hmax
// and hmin limits, and a fixed step never looks at the segment end (such a
// segment ends after nmax attempts, -2).  Returns 0 to continue, 1 at the
// segment end (g.h then holds the carried step), -1 when h < hmin, -2 after
// more than nmax attempts.
__device__ __forceinline__ int ext_attempt(Seg& g, const SetParams& P, double& Sx, double& Sy, double& Sz) {
  g.nstep++;
  if (g.nstep > P.nmax) return -2;
  g.acc = false;
  const double endDt = g.xf - g.x;
  double h = g.h;
  g.lastH = h;
  bool stop = false;
  if (P.fixed) {
    h = P.h0;
  } else if (h >= endDt) {
    h = endDt;
    stop = true;
  } else if (h > P.hmax) {
    h = std_min(h, P.hmax);
  } else if (h < P.hmin) {
    return -1;
  }
  const double tx = g.x - g.t0;
  double w[3], e[3];
  if (P.integrator == 2)
    magnus_stages(g, P, tx, h, Sx, Sy, Sz, w, e);
  else if (P.integrator == 3)
    quat_stages<false>(g, P, tx, h, Sx, Sy, Sz, w, e);
  else if (P.integrator == 5)
    quat_stages<true>(g, P, tx, h, Sx, Sy, Sz, w, e);
  else
    rkf45_stages(g, P, tx, h, Sx, Sy, Sz, w, e);
  double error = sqrt(fma(e[2], e[2], fma(e[1], e[1], e[0] * e[0])));
  error = std_max(error, 1.0e-16);
  const double ratio = P.rtol / error;
  const double lnr = log(ratio);
  double q = exp(rk45::E1 * lnr + rk45::E2 * g.lnprev);  // ratio^E1 * prev_ratio^E2
  q = std_min(q, 4.0);
  if ((q > 0.81 && error < 2.0 * P.rtol) || P.fixed) {
    g.acc = true;  // read by the adjoint's tape writer
    g.hu = h;
    g.turns += count_turn(Sy, Sz, w[1], w[2]);
    Sx = w[0]; Sy = w[1]; Sz = w[2];
    g.x += h;
    if (stop) {
      g.h = g.lastH;
      return 1;
    }
  }
  g.h = P.fixed ? h : h * q;
  g.lnprev = lnr;
  return 0;
}

}  // namespace st
