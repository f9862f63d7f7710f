/*
 * ORACLE — test infrastructure only (see spin_oracle.h).  CPU restatement of the
 * reference Spin-tracking hot path.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load this; the product never does.
 *
 * Build: make -C oracle port   (gcc -O2 -ffp-contract=off -fopenmp)
 *
 * Evaluation order of every double expression follows the reference source so
 * the results are bit-identical to the reference CPU build on the same host.
 * File:line citations are relative to the reference repository root.
 */
#include "spin_oracle.h"

#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* include/options.h:7-8 */
static const double OR_G = -9.81;
static const double OR_C2 = 299792458.0 * 299792458.0;

static or_counters *g_counters = NULL;
void or_set_counters(or_counters *c) { g_counters = c; }

/* Frozen accepted-step log (finite-difference checks of the adjoint): mode 1
 * appends every accepted step (h, last) of DOP853 and of integrator types 2-5 to the log; mode 2 replays the
 * log instead of the step controller (every step accepted with the logged h).
 * Runs that use the log must be single-threaded. */
static double *g_log = NULL;
static int64_t g_log_cap = 0, g_log_n = 0;
static int g_log_mode = 0;
void or_set_step_log(double *buf, int64_t cap, int mode) {
  g_log = buf;
  g_log_cap = cap;
  g_log_n = 0;
  g_log_mode = mode;
}
int64_t or_step_log_count(void) { return g_log_n; }

/* ------------------------------------------------------ elementary functions
 * The trajectory's log, acos, sin and cos: gas clocks -tc log(1 - u)
 * (src/particle.cpp:117-119), Marsaglia normals sqrt(-2 log s / s) (:89-107)
 * and cosine-law reflections acos(sqrt u), cos and sin (:309-328).
 *   mode 0 (default): the host C library, as the reference build calls it;
 *   mode 1: the correctly rounded double, evaluated in IEEE binary128
 *     (long double where it is binary128, else __float128 with libquadmath)
 *     and rounded once.  The binary128 results are within a few units of
 *     2^-113 relative, so the final rounding errs only where the exact value
 *     lies that close to a midpoint between doubles (~2^-58 of arguments);
 *   mode 2: the host C library;
 *   mode 3: correctly rounded except at one call per particle, the k-th
 *     (from 0, k per particle from or_set_math_pick) of those whose host
 *     library result is not the correctly rounded one, which takes the host
 *     library's result: it isolates the effect of a single last-bit
 *     difference on a trajectory.
 * In modes 1-3 each call is audited (or_set_math_audit): per particle the
 * number of calls whose two results differ and, for the first of them (in
 * mode 3 the picked one), the particle's time, the function and the
 * argument.
 * Test infrastructure for explaining the last-bit differences between the
 * reference's trajectories and ones computed with correctly rounded
 * functions; the reference's own results are mode 0. */
#if defined(__LDBL_MANT_DIG__) && __LDBL_MANT_DIG__ == 113
typedef long double or_quad;
#define Q_LOG logl
#define Q_ACOS acosl
#define Q_SIN sinl
#define Q_COS cosl
#else
#include <quadmath.h>
typedef __float128 or_quad;
#define Q_LOG logq
#define Q_ACOS acosq
#define Q_SIN sinq
#define Q_COS cosq
#endif

static int g_math_mode = 0;
static int64_t *g_audit_count = NULL;
static double *g_audit_t = NULL, *g_audit_arg = NULL;
static int *g_audit_fn = NULL;
static int g_audit_n = 0;
static const int64_t *g_pick = NULL;
static _Thread_local int tl_part = -1;     /* local slot of the particle being advanced */
static _Thread_local double tl_time = 0.0; /* its time at the start of the current segment */

void or_set_math_mode(int mode) { g_math_mode = mode; }
void or_set_math_pick(const int64_t *k) { g_pick = k; }
void or_set_math_audit(int64_t *count, double *first_t, int *first_fn, double *first_arg, int n) {
  g_audit_count = count;
  g_audit_t = first_t;
  g_audit_fn = first_fn;
  g_audit_arg = first_arg;
  g_audit_n = count ? n : 0;
}

static double cr_eval(int fn, double x) {
  const or_quad q = (or_quad)x;
  switch (fn) {
    case OR_FN_LOG: return (double)Q_LOG(q);
    case OR_FN_SIN: return (double)Q_SIN(q);
    case OR_FN_COS: return (double)Q_COS(q);
    default: return (double)Q_ACOS(q);
  }
}
static double libm_eval(int fn, double x) {
  switch (fn) {
    case OR_FN_LOG: return log(x);
    case OR_FN_SIN: return sin(x);
    case OR_FN_COS: return cos(x);
    default: return acos(x);
  }
}
static double tr_fn(int fn, double x) {
  if (g_math_mode == 0) return libm_eval(fn, x);
  const double c = cr_eval(fn, x);
  const double r = libm_eval(fn, x);
  if (r != c && !(r != r && c != c)) {
    const int i = tl_part;
    if (i >= 0 && i < g_audit_n) {
      const int64_t k = g_audit_count[i]++;
      const int picked = g_math_mode == 3 && g_pick && g_pick[i] == k;
      if (k == 0 || picked) { /* mode 3 records the picked call instead of the first */
        g_audit_t[i] = tl_time;
        g_audit_fn[i] = fn;
        g_audit_arg[i] = x;
      }
      if (picked) return r;
    }
  }
  return g_math_mode == 2 ? r : c;
}
static double tr_log(double x) { return tr_fn(OR_FN_LOG, x); }
static double tr_acos(double x) { return tr_fn(OR_FN_ACOS, x); }
static double tr_sin(double x) { return tr_fn(OR_FN_SIN, x); }
static double tr_cos(double x) { return tr_fn(OR_FN_COS, x); }

void or_math_eval(int fn, int mode, const double *x, double *y, int64_t n, int nthreads) {
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(static)
#endif
  for (int64_t k = 0; k < n; ++k) y[k] = mode ? cr_eval(fn, x[k]) : libm_eval(fn, x[k]);
}

/* ---------------------------------------------------------------- vec3 ops
 * Component-wise restatements of the reference `coords` operators
 * (src/double3.cpp:21-145).  Each returns a new value; order is preserved. */
static inline or_vec3 v3(double x, double y, double z) { or_vec3 r = {x, y, z}; return r; }
static inline or_vec3 vadd(or_vec3 a, or_vec3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline or_vec3 vsub(or_vec3 a, or_vec3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline or_vec3 vscale(double s, or_vec3 a) { return v3(a.x * s, a.y * s, a.z * s); }
static inline or_vec3 vdivs(or_vec3 a, double s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline or_vec3 vdiv(or_vec3 a, or_vec3 b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline or_vec3 vmul(or_vec3 a, or_vec3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline or_vec3 vcross(or_vec3 a, or_vec3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline double vdot(or_vec3 a, or_vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double vsum(or_vec3 a) { return a.x + a.y + a.z; }
static inline double vlen(or_vec3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline or_vec3 vfabs(or_vec3 a) { return v3(fabs(a.x), fabs(a.y), fabs(a.z)); }
static inline double dmax(double a, double b) { return (a > b) ? a : b; } /* max_d, src/integrator.cpp:30 */
static inline double dmin(double a, double b) { return (a < b) ? a : b; } /* min_d, src/integrator.cpp:25 */
static inline double std_min(double a, double b) { return (b < a) ? b : a; } /* std::min */
static inline double std_max(double a, double b) { return (a < b) ? b : a; } /* std::max */
static inline or_vec3 vmax(or_vec3 a, or_vec3 b) { return v3(dmax(a.x, b.x), dmax(a.y, b.y), dmax(a.z, b.z)); }
/* sgn with sgn(0) = +1, src/particle.cpp:24-31 */
static inline double sgn1(double v) { return (v < 0) ? -1.0 : 1.0; }

/* ------------------------------------------------------------ options */
size_t or_options_size(void) { return sizeof(or_options); }

void or_options_default(or_options *o) {
  /* defaults of include/options.h:11-60 */
  memset(o, 0, sizeof(*o));
  o->B0 = v3(3e-6, 0.0, 0.0);
  o->E = v3(75e5, 0.0, 0.0);
  o->L = v3(0.07, 0.1, 0.4);
  o->yi = v3(0.0, 0.0, 1.0);
  o->m = 1.20239e-26;
  o->t0 = 0.0;
  o->tf = 10.0;
  o->rtol = 1e-12;
  o->atol = 1e-12;
  o->beta = 0.0;
  o->uround = 1e-16;
  o->safe = 0.9;
  o->fac1 = 0.333;
  o->fac2 = 6.0;
  o->hmax = 1.0;
  o->hmin = 1.0e-8;
  o->h = 0.001;
  o->T = 4.2;
  o->gamma = -2.038e8;
  o->V = 5.0;
  o->swapStepSize = 1.0 - 4; /* sic: the reference default is -3 */
  o->maxPosStep = 0.1;
  o->ioutInt = 0.05;
  o->diffuse = 1.0;
  o->nmax = 10000000u;
  o->seed = 0u;
  o->integratorType = 0;
  o->numParticles = 1000;
  o->numPerGPUBlock = 128;
  o->iout = 2;
  o->dist = 'C';
  o->gas_coll = true;
  o->gravity = true;
  o->fixedStepSize = false;
  o->keepStepSize = false;
}

/* Split on ',' and drop every whitespace character of each token
 * (grabElementsInLine / removeWhitespace, src/optionsParser.cpp:11-37). */
#define OR_MAX_TOK 16
#define OR_TOK_LEN 256
static int split_line(const char *s, char tok[OR_MAX_TOK][OR_TOK_LEN]) {
  int n = 0, len = 0;
  tok[0][0] = 0;
  for (const char *c = s;; ++c) {
    if (*c == ',' || *c == 0) {
      tok[n][len] = 0;
      ++n;
      if (*c == 0 || n >= OR_MAX_TOK) break;
      len = 0;
      tok[n][0] = 0;
    } else if (!isspace((unsigned char)*c)) {
      if (len < OR_TOK_LEN - 1) tok[n][len++] = *c;
    }
  }
  return n;
}

/* std::stod semantics on a whitespace-free token (leading number parsed). */
static double tok_d(const char *t) { return strtod(t, NULL); }
static long tok_i(const char *t) { return strtol(t, NULL, 10); }
/* to_bool (src/optionsParser.cpp:16-22): boolalpha extraction of the lowered token,
 * so only a leading "true" (any case) parses true; "1" fails and gives false. */
static bool tok_b(const char *t) {
  char low[OR_TOK_LEN];
  size_t i = 0;
  for (; t[i] && i < sizeof(low) - 1; ++i) low[i] = (char)tolower((unsigned char)t[i]);
  low[i] = 0;
  if (!strncmp(low, "true", 4)) return true;
  if (!strncmp(low, "false", 5)) return false;
  /* boolalpha extraction of anything else fails and leaves false */
  return false;
}

int or_parse_line(or_options *o, const char *line) {
  char tok[OR_MAX_TOK][OR_TOK_LEN];
  int n = split_line(line, tok);
  if (n < 2) return -1; /* "Misunderstood input line", src/optionsParser.cpp:44-48 */
  const char *k = tok[0];
#define VEC3(name, field)                                                             \
  if (!strcmp(k, name)) {                                                            \
    if (n < 4) return -2;                                                            \
    o->field = v3(tok_d(tok[1]), tok_d(tok[2]), tok_d(tok[3]));                      \
    return 0;                                                                        \
  }
#define DBL(name, field) if (!strcmp(k, name)) { o->field = tok_d(tok[1]); return 0; }
#define INT(name, field) if (!strcmp(k, name)) { o->field = (int)tok_i(tok[1]); return 0; }
#define UNS(name, field) if (!strcmp(k, name)) { o->field = (unsigned int)(int)tok_i(tok[1]); return 0; }
#define BOOL(name, field) if (!strcmp(k, name)) { o->field = tok_b(tok[1]); return 0; }
  VEC3("L", L) VEC3("yi", yi) VEC3("Gx", Gx) VEC3("Gy", Gy) VEC3("Gz", Gz)
  if (!strcmp(k, "dist")) { o->dist = tok[1][0]; return 0; }
  DBL("m", m) BOOL("gas_coll", gas_coll) DBL("T", T) DBL("diffuse", diffuse) DBL("gamma", gamma)
  DBL("V", V) DBL("a", a) DBL("w", w) BOOL("gravity", gravity) BOOL("fixedStepSize", fixedStepSize)
  BOOL("keepStepSize", keepStepSize) VEC3("B0", B0) VEC3("E", E) DBL("t0", t0) DBL("tf", tf)
  DBL("rtol", rtol) DBL("atol", atol) DBL("beta", beta) DBL("uround", uround) DBL("safe", safe)
  DBL("fac1", fac1) DBL("fac2", fac2) DBL("hmax", hmax) DBL("hmin", hmin) DBL("h", h)
  UNS("nmax", nmax) UNS("seed", seed) DBL("maxPosStep", maxPosStep) INT("integratorType", integratorType)
  DBL("swapStepSize", swapStepSize) INT("numParticles", numParticles) INT("numPerGPUBlock", numPerGPUBlock)
  DBL("ioutInt", ioutInt) INT("iout", iout)
#undef VEC3
#undef DBL
#undef INT
#undef UNS
#undef BOOL
  return 1; /* "Unrecognized Option ... Line Ignored", src/optionsParser.cpp:171-174 */
}

int or_parse_file(const char *path, or_options *o) {
  or_options_default(o);
  FILE *f = fopen(path, "r");
  if (!f) return 1; /* the reference silently keeps the defaults */
  char line[4096];
  while (fgets(line, sizeof(line), f)) {
    size_t L = strlen(line);
    while (L && (line[L - 1] == '\n' || line[L - 1] == '\r')) line[--L] = 0;
    or_parse_line(o, line);
  }
  fclose(f);
  return 0;
}

void or_derive(or_options *o) {
  const double k = 1.380649e-23; /* src/simulation.cpp:9-11 */
  o->tc = 1.6e-4 * o->m / (k * pow(o->T, 8.0));
  o->sqrtKT_m = sqrt(k * o->T / o->m);
}

/* ---------------------------------------------------------------- RNG
 * Seeding: two splitmix64 outputs of the 32-bit sum seed + ipart, each split into 32-bit
 * halves, then three discarded draws (src/particle.cpp:648-663). */
static uint64_t splitmix_next(uint64_t *s) {
  uint64_t r = (*s += 0x9E3779B97F4A7C15ull);
  r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
  r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
  return r ^ (r >> 31);
}

void or_rng_seed(or_rng *r, unsigned int seed, unsigned int ipart) {
  /* opt.seed + ipart is an unsigned int sum: it wraps at 2^32 */
  uint64_t s = (uint64_t)(uint32_t)(seed + ipart);
  uint64_t a = splitmix_next(&s);
  r->x = (uint32_t)a;
  r->y = (uint32_t)(a >> 32);
  uint64_t b = splitmix_next(&s);
  r->z = (uint32_t)b;
  r->w = (uint32_t)(b >> 32);
  r->spare = 0.0;
  r->has_spare = false;
  or_uniform(r);
  or_uniform(r);
  or_uniform(r);
}

/* The reference's own xoshiro256+ variant (src/particle.cpp:59-70): output
 * x + z, and the last word is re-derived from z rather than rotated in place.
 * (The unused include/rng.h holds the textbook form; parity needs this one.) */
uint64_t or_xoshiro(or_rng *r) {
  const uint64_t out = r->x + r->z;
  const uint64_t t = r->y << 17;
  r->z ^= r->x;
  r->w ^= r->y;
  r->y ^= r->z;
  r->x ^= r->w;
  r->z ^= t;
  r->w = (r->z << 45) | (r->z >> 19);
  return out;
}

/* src/particle.cpp:72-87: top 53 bits scaled by 2^-53 */
double or_uniform(or_rng *r) { return (double)(or_xoshiro(r) >> 11) * 0x1.0p-53; }
static double or_uniform_ab(or_rng *r, double lo, double hi) { return or_uniform(r) * (hi - lo) + lo; }

/* Marsaglia polar method with the second value cached (src/particle.cpp:89-107). */
double or_normal(or_rng *r, double mean, double std) {
  if (r->has_spare) {
    r->has_spare = false;
    return r->spare * std + mean;
  }
  double u, v, s;
  do {
    u = or_uniform_ab(r, -1.0, 1.0);
    v = or_uniform_ab(r, -1.0, 1.0);
    s = u * u + v * v;
  } while (s >= 1.0 || s == 0.0);
  s = sqrt(-2.0 * tr_log(s) / s);
  r->spare = v * s;
  r->has_spare = true;
  return mean + std * u * s;
}

static double or_maxboltz(or_rng *r, double sq) { return or_normal(r, 0.0, 1.0) * sq; } /* :109-111 */
static double or_unif02pi(or_rng *r) { return or_uniform(r) * 2.0 * M_PI; }          /* :113-115 */
double or_exponential(or_rng *r, double tc) { return -tc * tr_log(1.0 - or_uniform(r)); } /* :117-119 */

/* ------------------------------------------------------------ particles */
int or_particles_alloc(or_particles *p, int n) {
  memset(p, 0, sizeof(*p));
  p->n = n;
  size_t m = n > 0 ? (size_t)n : 1;
#define AL(f) if (!(p->f = calloc(m, sizeof(*p->f)))) return -1;
  AL(S) AL(v) AL(v_old) AL(pos) AL(pos_old) AL(t) AL(t_old) AL(h) AL(next_gas) AL(rng) AL(fail)
  AL(n_bounce) AL(n_coll) AL(n_steps) AL(stop) AL(coll_type) AL(wall_hit)
#undef AL
  return 0;
}

void or_particles_free(or_particles *p) {
  free(p->spec);
  free(p->S); free(p->v); free(p->v_old); free(p->pos); free(p->pos_old); free(p->t); free(p->t_old);
  free(p->h); free(p->next_gas); free(p->rng); free(p->fail); free(p->n_bounce); free(p->n_coll);
  free(p->n_steps); free(p->stop); free(p->coll_type); free(p->wall_hit);
  memset(p, 0, sizeof(*p));
}

/* initParticlesCPU (src/particle.cpp:638-710) for local slots 0..n-1 holding
 * global particle indices first_index.. (the seed uses the global index). */
void or_init(const or_options *o, or_particles *p, int first_index) {
  for (int i = 0; i < p->n; ++i) {
    tl_part = i;
    tl_time = o->t0;
    or_rng r;
    or_rng_seed(&r, o->seed, (unsigned int)(first_index + i));
    or_vec3 pos;
    pos.x = or_uniform(&r) * o->L.x - o->L.x / 2.0;
    pos.y = or_uniform(&r) * o->L.y - o->L.y / 2.0;
    pos.z = or_uniform(&r) * o->L.z - o->L.z / 2.0;
    p->pos[i] = pos;
    p->pos_old[i] = pos;
    p->next_gas[i] = o->gas_coll ? or_exponential(&r, o->tc) : DBL_MAX;
    or_vec3 vel = v3(0.0, 0.0, 0.0);
    if (o->dist == 'C') {
      /* the CPU build always draws three normals, even for V == 0 */
      or_vec3 d;
      d.x = or_normal(&r, 0.0, 1.0);
      d.y = or_normal(&r, 0.0, 1.0);
      d.z = or_normal(&r, 0.0, 1.0);
      double nrm = vlen(d);
      vel = vdivs(vscale(o->V, d), nrm);
    } else if (o->dist == 'M') {
      vel.x = or_maxboltz(&r, o->sqrtKT_m);
      vel.y = or_maxboltz(&r, o->sqrtKT_m);
      vel.z = or_maxboltz(&r, o->sqrtKT_m);
    }
    p->v[i] = vel;
    p->v_old[i] = vel;
    p->rng[i] = r;
    p->S[i] = o->yi;
    p->t[i] = o->t0;
    p->t_old[i] = o->t0;
    p->h[i] = o->h;
    p->stop[i] = false;
    p->coll_type[i] = 'W';
    p->wall_hit[i] = 0;
    p->fail[i] = 0;
    p->n_bounce[i] = 0;
    p->n_coll[i] = 0;
    p->n_steps[i] = 0;
  }
  tl_part = -1;
}

/* ------------------------------------------------------------ field model
 * interpolate (src/integrator.cpp:48-61) */
void or_interpolate(const or_options *o, double t, double t0, const or_vec3 *p_old, const or_vec3 *v_old,
                    or_vec3 *p_out, or_vec3 *v_out) {
  if (o->gravity) {
    const or_vec3 a = v3(0.0, OR_G, 0.0);
    *p_out = vadd(vadd(*p_old, vscale(t - t0, *v_old)), vscale(t - t0, vscale(t - t0, vscale(0.5, a))));
    *v_out = vadd(*v_old, vscale(t - t0, a));
  } else {
    *p_out = vadd(*p_old, vscale(t - t0, *v_old));
    *v_out = *v_old;
  }
}

/* Bloch right-hand side f = y x gamma*B(t) with
 * B = pulse(t) + B0 + cross(v,E)/c^2 + grad(pos)  (src/integrator.cpp:40-46, 63-70, 83-88). */
static or_vec3 bloch(const or_options *o, double t, or_vec3 y, double t0, const or_vec3 *p_old,
                     const or_vec3 *v_old) {
  or_vec3 p, v;
  or_interpolate(o, t, t0, p_old, v_old, &p, &v);
  or_vec3 G = v3(vdot(p, o->Gx), vdot(p, o->Gy), vdot(p, o->Gz));
  or_vec3 pulse = v3(0.0, 0.0, o->a * cos(o->w * t));
  or_vec3 B = vadd(vadd(vadd(pulse, o->B0), vscale(1.0 / OR_C2, vcross(v, o->E))), G);
  return vcross(y, vscale(o->gamma, B));
}

/* ------------------------------------------------------------ DOP853
 * Hairer's DOP853 tableau, values of include/coeff.h:6-176 written as
 * shortest round-trip doubles. */
enum { DC2, DC3, DC4, DC5, DC6, DC7, DC8, DC9, DC10, DC11 };
static const double dop_c[10] = {0.05260015195876773, 0.0789002279381516, 0.1183503419072274, 0.2816496580927726, 0.3333333333333333, 0.25, 0.3076923076923077, 0.6512820512820513, 0.6, 0.8571428571428571};
/* Stage rows: (k slot, coefficient) in the reference's summation order.  Slots
 * 1..10 are k1..k10; stage 11 writes slot 2 and stage 12 slot 3, as the
 * reference reuses k2/k3 (src/integrator.cpp:176-183). */
typedef struct { int n; int slot[9]; double a[9]; } dop_row;
static const dop_row dop_rows[11] = {
    {1, {1}, {0.05260015195876773}},
    {2, {1, 2}, {0.0197250569845379, 0.0591751709536137}},
    {2, {1, 3}, {0.02958758547680685, 0.08876275643042054}},
    {3, {1, 3, 4}, {0.2413651341592667, -0.8845494793282861, 0.924834003261792}},
    {3, {1, 4, 5}, {0.037037037037037035, 0.17082860872947386, 0.12546768756682242}},
    {4, {1, 4, 5, 6}, {0.037109375, 0.17025221101954405, 0.06021653898045596, -0.017578125}},
    {5, {1, 4, 5, 6, 7}, {0.03709200011850479, 0.17038392571223998, 0.10726203044637328, -0.015319437748624402, 0.008273789163814023}},
    {6, {1, 4, 5, 6, 7, 8}, {0.6241109587160757, -3.3608926294469414, -0.868219346841726, 27.59209969944671, 20.154067550477894, -43.48988418106996}},
    {7, {1, 4, 5, 6, 7, 8, 9}, {0.47766253643826434, -2.4881146199716677, -0.590290826836843, 21.230051448181193, 15.279233632882423, -33.28821096898486, -0.020331201708508627}},
    {8, {1, 4, 5, 6, 7, 8, 9, 10}, {-0.9371424300859873, 5.186372428844064, 1.0914373489967295, -8.149787010746927, -18.52006565999696, 22.739487099350505, 2.4936055526796523, -3.0467644718982196}},
    {9, {1, 4, 5, 6, 7, 8, 9, 10, 2}, {2.273310147516538, -10.53449546673725, -2.0008720582248625, -17.9589318631188, 27.94888452941996, -2.8589982771350235, -8.87285693353063, 12.360567175794303, 0.6433927460157636}},
};
/* 8th-order weights over slots (1,6,7,8,9,10,2,3) and the two error rows. */
static const int dop_bslot[8] = {1, 6, 7, 8, 9, 10, 2, 3};
static const double dop_b[8] = {0.054293734116568765, 4.450312892752409, 1.8915178993145003, -5.801203960010585, 0.3111643669578199, -0.1521609496625161, 0.20136540080403034, 0.04471061572777259};
static const double dop_bhh[3] = {0.2440944881889764, 0.7338466882816118, 0.022058823529411766};
static const double dop_er[8] = {0.01312004499419488, -1.2251564463762044, -0.4957589496572502, 1.6643771824549864, -0.35032884874997366, 0.3341791187130175, 0.08192320648511571, -0.022355307863886294};

static or_vec3 lincomb(int n, const int *slot, const double *a, const or_vec3 *k) {
  or_vec3 s = vscale(a[0], k[slot[0]]);
  for (int j = 1; j < n; ++j) s = vadd(s, vscale(a[j], k[slot[j]]));
  return s;
}

/* integrateDOP (src/integrator.cpp:90-249).  h in: first trial step;
 * h out: the (possibly truncated) last accepted step.  Returns 1, or -1 when
 * more than nmax attempts were needed. */
int or_integrate_dop(const or_options *o, double t0, double tf, or_vec3 *yio, const or_vec3 *p_old,
                     const or_vec3 *v_old, double *hio) {
  or_vec3 k[11];
  or_vec3 y = *yio;
  double h = *hio;
  unsigned int nstep = 0, naccpt = 0;
  double x = t0, xf = tf;
  double facold = 1.0e-4;
  const double expo1 = 1.0 / 8.0 - o->beta * 0.2;
  const double facc1 = 1.0 / o->fac1, facc2 = 1.0 / o->fac2;
  const double posneg = (tf - t0 < 0.0) ? -fabs(1.0) : fabs(1.0);
  int last = 0, reject = 0;
  k[1] = bloch(o, x, y, t0, p_old, v_old);
  for (;;) {
    if (nstep > o->nmax) {
      *yio = y;
      *hio = h;
      return -1;
    }
    if (g_log_mode == 2) { /* replay: the logged accepted step */
      if (g_log_n >= g_log_cap) {
        *yio = y;
        return -9;
      }
      h = g_log[2 * g_log_n];
      last = g_log[2 * g_log_n + 1] != 0.0;
      g_log_n++;
    } else {
      if ((x + 1.01 * h - xf) * posneg > 0.0) {
        h = xf - x;
        last = 1;
      }
      if (h < o->hmin && last != 1) h = o->hmin;
    }
    nstep++;
    if (g_counters) {
#pragma omp atomic
      g_counters->dop_attempts++;
    }
    /* stage 2 groups (h*a21)*k1; the later stages h*(sum) */
    or_vec3 yy = vadd(y, vscale(h * dop_rows[0].a[0], k[1]));
    k[2] = bloch(o, x + dop_c[DC2] * h, yy, t0, p_old, v_old);
    const int out_slot[10] = {3, 4, 5, 6, 7, 8, 9, 10, 2, 3};
    for (int s = 1; s < 11; ++s) {
      yy = vadd(y, vscale(h, lincomb(dop_rows[s].n, dop_rows[s].slot, dop_rows[s].a, k)));
      double ts = (s == 10) ? (x + h) : (x + dop_c[s] * h);
      k[out_slot[s - 1]] = bloch(o, ts, yy, t0, p_old, v_old);
    }
    double xph = x + h;
    or_vec3 k4 = lincomb(8, dop_bslot, dop_b, k);
    or_vec3 k5 = vadd(y, vscale(h, k4));
    /* atol + rtol*max(|y|,|y_new|), component-wise */
    or_vec3 sk = v3(o->atol + o->rtol * dmax(fabs(y.x), fabs(k5.x)), o->atol + o->rtol * dmax(fabs(y.y), fabs(k5.y)),
            o->atol + o->rtol * dmax(fabs(y.z), fabs(k5.z)));
    or_vec3 e1 = vsub(vsub(vsub(k4, vscale(dop_bhh[0], k[1])), vscale(dop_bhh[1], k[9])), vscale(dop_bhh[2], k[3]));
    or_vec3 q = vdiv(e1, sk);
    double err2 = 0.0 + vsum(vmul(q, q));
    or_vec3 e2 = lincomb(8, dop_bslot, dop_er, k);
    q = vdiv(e2, sk);
    double err = 0.0 + vsum(vmul(q, q));
    double deno = err + 0.01 * err2;
    if (deno <= 0.0) deno = 1.0;
    err = fabs(h) * err * sqrt(1.0 / (deno * 3.0));
    double fac11 = pow(err, expo1);
    double fac = fac11 / pow(facold, o->beta);
    fac = dmax(facc2, dmin(facc1, fac / o->safe));
    double hnew = h / fac;
    if (err <= 1.0 || o->fixedStepSize || g_log_mode == 2) {
      if (g_log_mode == 1 && g_log_n < g_log_cap) {
        g_log[2 * g_log_n] = h;
        g_log[2 * g_log_n + 1] = last ? 1.0 : 0.0;
        g_log_n++;
      }
      facold = dmax(err, 1.0e-4);
      naccpt++;
      k[1] = bloch(o, xph, k5, t0, p_old, v_old);
      y = k5;
      x = xph;
      if (last) {
        *yio = y;
        *hio = h;
        return 1;
      }
      if (fabs(hnew) > o->hmax) hnew = posneg * o->hmax;
      if (reject) hnew = posneg * dmin(fabs(hnew), fabs(h));
      reject = 0;
    } else {
      hnew = h / dmin(facc1, fac11 / o->safe);
      reject = 1;
      last = 0;
    }
    if (!o->fixedStepSize) h = hnew;
  }
}

/* ------------------------------------------------------------ RK45
 * Tableau of include/coeff.h:178-218 (RK4(5) with the 2/9, 1/3, 3/4, 1, 5/6 nodes). */
static const double rk_A[7] = {0.0, 0.0, 0.2222222222222222, 0.3333333333333333, 0.75, 1.0, 0.8333333333333334};
static const double rk_B21 = 0.2222222222222222;
static const double rk_B3[2] = {0.08333333333333333, 0.25};
static const double rk_B4[3] = {0.5390625, -1.8984375, 2.109375};
static const double rk_B5[4] = {-1.4166666666666667, 6.75, -5.4, 1.0666666666666667};
static const double rk_B6[5] = {0.15046296296296297, -0.3125, 0.8125, 0.14814814814814814, 0.034722222222222224};
static const double rk_CH[6] = {0.10444444444444445, 0.0, 0.48, 0.14222222222222222, 0.03333333333333333, 0.24};
static const double rk_CT[6] = {0.006666666666666667, 0.0, -0.03, 0.21333333333333335, 0.05, -0.24};

/* integrateRK45 (src/integrator.cpp:251-337), including its first-stage
 * quirk: k1 is evaluated at the previous attempt's last stage state (zero on
 * the first attempt of a call), not at y.  Returns 0, -1 (h < hmin) or
 * -2 (more than nmax attempts). */
int or_integrate_rk45(const or_options *o, double t0, double tf, or_vec3 *yio, const or_vec3 *p_old,
                      const or_vec3 *v_old, double *hio) {
  or_vec3 y = *yio, yy = v3(0.0, 0.0, 0.0), k[7];
  double h = *hio, t = t0, lastH = h, prev_ratio = 1.0;
  int stop = 0, nstep = 0;
  const double e1 = 0.7 / 7.0, e2 = -0.4 / 7.0;
  for (;;) {
    nstep++;
    if ((unsigned int)nstep > o->nmax) {
      *yio = y;
      *hio = h;
      return -2;
    }
    if (g_counters) {
#pragma omp atomic
      g_counters->rk45_attempts++;
    }
    double endDt = tf - t;
    lastH = h;
    if (o->fixedStepSize) {
      h = o->h;
    } else {
      if (h > o->hmax) {
        h = std_min(h, o->hmax);
      } else if (h < o->hmin) {
        *yio = y;
        *hio = h;
        return -1;
      }
    }
    if (h >= endDt) {
      h = endDt;
      stop = 1;
    } else {
      lastH = h;
      stop = 0;
    }
    k[1] = bloch(o, t, yy, t0, p_old, v_old);
    yy = vadd(y, vscale(h * rk_B21, k[1]));
    k[2] = bloch(o, t + rk_A[2] * h, yy, t0, p_old, v_old);
    yy = vadd(vadd(y, vscale(h * rk_B3[0], k[1])), vscale(h * rk_B3[1], k[2]));
    k[3] = bloch(o, t + rk_A[3] * h, yy, t0, p_old, v_old);
    yy = y;
    for (int j = 0; j < 3; ++j) yy = vadd(yy, vscale(h * rk_B4[j], k[1 + j]));
    k[4] = bloch(o, t + rk_A[4] * h, yy, t0, p_old, v_old);
    yy = y;
    for (int j = 0; j < 4; ++j) yy = vadd(yy, vscale(h * rk_B5[j], k[1 + j]));
    k[5] = bloch(o, t + rk_A[5] * h, yy, t0, p_old, v_old);
    yy = y;
    for (int j = 0; j < 5; ++j) yy = vadd(yy, vscale(h * rk_B6[j], k[1 + j]));
    k[6] = bloch(o, t + rk_A[6] * h, yy, t0, p_old, v_old);
    or_vec3 wsum = vscale(rk_CH[0], k[1]);
    for (int j = 1; j < 6; ++j) wsum = vadd(wsum, vscale(rk_CH[j], k[1 + j]));
    or_vec3 step = vadd(y, vscale(h, wsum));
    or_vec3 te = vscale(rk_CT[0], k[1]);
    for (int j = 1; j < 6; ++j) te = vadd(te, vscale(rk_CT[j], k[1 + j]));
    te = vscale(h, te);
    double error = std_max(vlen(te), 1.0e-16);
    double tol = o->rtol;
    double ratio = tol / error;
    double q = pow(ratio, e1) * pow(prev_ratio, e2);
    q = std_min(q, 4.0);
    if ((q > 0.81 && error < 2 * tol) || o->fixedStepSize) {
      y = step;
      t += h;
      if (stop) {
        *yio = y;
        *hio = lastH;
        return 0;
      }
    } else {
      if (stop) stop = 0;
    }
    if (!o->fixedStepSize) h = h * q;
    prev_ratio = ratio;
  }
}

/* ------------------------------------------------------------ integrator types 2-5
 * Tableaux of include/coeff.h:220-320 (RKF45COEF, CFET8, CFET6, GL5) as
 * shortest round-trip doubles (identical bits). */
static const double rkf_A[7] = {0.0, 0.0, 0.25, 0.375, 0.9230769230769231, 1.0, 0.5};
static const double rkf_B21 = 0.25;
static const double rkf_B3[2] = {0.09375, 0.28125};
static const double rkf_B4[3] = {0.8793809740555303, -3.277196176604461, 3.3208921256258535};
static const double rkf_B5[4] = {2.0324074074074074, -8.0, 7.173489278752436, -0.20589668615984405};
static const double rkf_B6[5] = {-0.2962962962962963, 2.0, -1.3816764132553607, 0.4529727095516569, -0.275};
static const double rkf_C[6] = {0.11851851851851852, 0.0, 0.5189863547758284, 0.5061314903420167, -0.18,
                                0.03636363636363636};
static const double rkf_CR[6] = {0.11574074074074074, 0.0, 0.5489278752436647, 0.5353313840155945, -0.2, 0.0};
static const double rk_C5[5] = {0.1111111111111111, 0.0, 0.45, 0.35555555555555557, 0.08333333333333333};
/* CFET8 G[i][j] = G(i+1)(j+1), CFET6 H likewise, Gauss-Legendre nodes X */
static const double cfet8_G[6][5] = {
    {-0.005984812750244602, 0.020217897716672675, -0.03646660716686794, 0.04245408899634467, 0.14949496424802844},
    {0.02512881778391826, -0.08955337580937157, 0.19032828600393248, 0.28920194841768715, -0.03568486888016069},
    {-0.04972613261435144, 0.6572496090804754, 0.11725149008224456, -0.43611911073577403, 0.18080345083145516},
    {0.0464837870954061, -0.6265183532355708, -0.11144873822286155, 0.4154988625423615, -0.17224148557040517},
    {0.015567390500242426, -0.0677120111619075, -0.15241336773272682, -0.08803798509100481, -0.0013284996209207986},
    {-0.034049168494873015, 0.12263276452977083, 0.2699423185170027, 0.12263276452977094, -0.03404916849487304}};
static const double cfet6_H[3][5] = {
    {-0.007431519425246311, 0.022452824849980513, -0.03620393417193995, 0.0409779901800809, 0.1516046385671249},
    {0.03095749686312404, -0.10116885619385878, 0.1997455955716367, 0.3010242365525433, -0.055594729593982636},
    {-0.001072443882925378, -0.023971860139062367, -0.04263887835494916, -0.023971860139062388,
     -0.0010724438829253797}};
static const double gl5_X[5] = {0.046910077030668074, 0.2307653449471585, 0.5, 0.7692346550528415,
                                0.9530899229693319};

/* findCrossTerm (src/integrator.cpp:63-70): gamma * B at time t. */
static or_vec3 omega(const or_options *o, double t, double t0, const or_vec3 *p_old, const or_vec3 *v_old) {
  or_vec3 p, v;
  or_interpolate(o, t, t0, p_old, v_old, &p, &v);
  or_vec3 G = v3(vdot(p, o->Gx), vdot(p, o->Gy), vdot(p, o->Gz));
  or_vec3 pulse = v3(0.0, 0.0, o->a * cos(o->w * t));
  or_vec3 B = vadd(vadd(vadd(pulse, o->B0), vscale(1.0 / OR_C2, vcross(v, o->E))), G);
  return vscale(o->gamma, B);
}

/* Quaternions (w, x, y, z) of src/quaternion.cpp: qMult, qv_mult (v as the
 * pure quaternion (0, v), rotated as q v q*), rodriguezQuat and rodriguez. */
typedef struct { double w, x, y, z; } or_quat;
static or_quat qmul(or_quat a, or_quat b) {
  or_quat r;
  r.w = a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z;
  r.x = a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y;
  r.y = a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z;
  r.z = a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x;
  return r;
}
static or_vec3 qrotate(or_quat q, or_vec3 v) {
  or_quat p = {0.0, v.x, v.y, v.z}, qc = {q.w, -q.x, -q.y, -q.z};
  p = qmul(qmul(q, p), qc);
  return v3(p.x, p.y, p.z);
}
/* rotation by |k| dt about -k/|k|, as a unit quaternion */
static or_quat rot_quat(or_vec3 k, double dt) {
  double angle = vlen(k);
  or_vec3 n = vdivs(k, angle);
  double h = angle * dt;
  n = vscale(-sin(h / 2.0), n);
  or_quat r = {cos(h / 2.0), n.x, n.y, n.z};
  return r;
}
/* v rotated by the angle |k| about -k/|k| (Rodrigues' formula) */
static or_vec3 rodrigues(or_vec3 k, or_vec3 v) {
  const double angle = vlen(k);
  const double s = sin(angle);
  const double c = cos(angle);
  return vadd(vadd(vscale(c, v), vscale(s / angle, vcross(v, k))), vscale(vdot(k, v) * (1.0 - c) / (angle * angle), k));
}

/* (c[0] B[0] + ... + c[4] B[4]) h with the coefficients taken forwards, or
 * backwards (c[4] B[0] + ... + c[0] B[4]) when rev is set. */
static or_vec3 magnus_exponent(const double c[5], int rev, const or_vec3 B[5], double h) {
  or_vec3 s = vscale(c[rev ? 4 : 0], B[0]);
  for (int j = 1; j < 5; ++j) s = vadd(s, vscale(c[rev ? 4 - j : j], B[j]));
  return vscale(h, s);
}

/* One attempt's proposal (ws) and error vector (te) of types 2-5 at (t, y, h).
 * yy carries RKF45's stage state between attempts (its k1 quirk). */
static void ext_stages(const or_options *o, int type, double t, double h, or_vec3 y, or_vec3 *yy, double t0,
                       const or_vec3 *p_old, const or_vec3 *v_old, or_vec3 *ws, or_vec3 *te) {
  if (type == 2) {
    /* integrateMagnusCFET (src/integrator.cpp:670-698): the CFET8 product
     * applied from its 11th exponent inwards, and the CFET6 one beside it */
    or_vec3 B[5];
    for (int i = 0; i < 5; ++i) B[i] = omega(o, t + gl5_X[i] * h, t0, p_old, v_old);
    or_vec3 y8 = y;
    for (int r = 0; r < 5; ++r) y8 = rodrigues(magnus_exponent(cfet8_G[r], 1, B, h), y8);   /* k11 .. k7 */
    for (int r = 5; r >= 0; --r) y8 = rodrigues(magnus_exponent(cfet8_G[r], 0, B, h), y8);  /* k6 .. k1 */
    or_vec3 y6 = y;
    for (int r = 0; r < 2; ++r) y6 = rodrigues(magnus_exponent(cfet6_H[r], 1, B, h), y6);   /* k5, k4 */
    for (int r = 2; r >= 0; --r) y6 = rodrigues(magnus_exponent(cfet6_H[r], 0, B, h), y6);  /* k3 .. k1 */
    *ws = y8;
    *te = vsub(y8, y6);
  } else if (type == 3 || type == 5) {
    /* integrateRK45Quaternion (:476-497) / integrateRKF45Quaternion (:565-586):
     * the stage fields at the tableau's nodes, composed as rotations */
    const double *A = (type == 3) ? rk_A : rkf_A;
    const double *W = (type == 3) ? rk_CH : rkf_C;
    const double *E = (type == 3) ? rk_C5 : rkf_C;
    or_vec3 k[7];
    k[1] = omega(o, t, t0, p_old, v_old);
    for (int s = 2; s <= 6; ++s) k[s] = omega(o, t + A[s] * h, t0, p_old, v_old);
    or_quat qw = rot_quat(k[1], h * W[0]), qe = rot_quat(k[1], h * E[0]);
    for (int s = 2; s <= 6; ++s) qw = qmul(rot_quat(k[s], h * W[s - 1]), qw);
    for (int s = 2; s <= 5; ++s) qe = qmul(rot_quat(k[s], h * E[s - 1]), qe);
    *ws = qrotate(qw, y);
    *te = vsub(*ws, qrotate(qe, y));
  } else {
    /* integrateRKF45 (:384-396), with RK45's first-stage quirk */
    or_vec3 k[7];
    k[1] = bloch(o, t, *yy, t0, p_old, v_old);
    *yy = vadd(y, vscale(h * rkf_B21, k[1]));
    k[2] = bloch(o, t + rkf_A[2] * h, *yy, t0, p_old, v_old);
    *yy = vadd(vadd(y, vscale(h * rkf_B3[0], k[1])), vscale(h * rkf_B3[1], k[2]));
    k[3] = bloch(o, t + rkf_A[3] * h, *yy, t0, p_old, v_old);
    *yy = y;
    for (int j = 0; j < 3; ++j) *yy = vadd(*yy, vscale(h * rkf_B4[j], k[1 + j]));
    k[4] = bloch(o, t + rkf_A[4] * h, *yy, t0, p_old, v_old);
    *yy = y;
    for (int j = 0; j < 4; ++j) *yy = vadd(*yy, vscale(h * rkf_B5[j], k[1 + j]));
    k[5] = bloch(o, t + rkf_A[5] * h, *yy, t0, p_old, v_old);
    *yy = y;
    for (int j = 0; j < 5; ++j) *yy = vadd(*yy, vscale(h * rkf_B6[j], k[1 + j]));
    k[6] = bloch(o, t + rkf_A[6] * h, *yy, t0, p_old, v_old);
    or_vec3 wsum = vscale(rkf_C[0], k[1]), tsum = vscale(rkf_CR[0], k[1]);
    for (int j = 1; j < 6; ++j) wsum = vadd(wsum, vscale(rkf_C[j], k[1 + j]));
    for (int j = 1; j < 6; ++j) tsum = vadd(tsum, vscale(rkf_CR[j], k[1 + j]));
    *ws = vadd(y, vscale(h, wsum));
    *te = vscale(h, tsum);  /* the whole fourth-order increment, as the reference has it */
  }
}

/* integrateMagnusCFET (src/integrator.cpp:625-722), integrateRK45Quaternion
 * (:441-528), integrateRKF45 (:339-439) and integrateRKF45Quaternion
 * (:530-623), selected by o->integratorType 2, 3, 4, 5.  Their shared step
 * controller differs from RK45's: the segment end is tested before the
 * hmax/hmin limits, and a fixed step never looks at the segment end (such a
 * run ends after nmax attempts, -2).  Returns 0, -1 (h < hmin) or -2. */
int or_integrate_ext(const or_options *o, double t0, double tf, or_vec3 *yio, const or_vec3 *p_old,
                     const or_vec3 *v_old, double *hio) {
  const int type = o->integratorType;
  or_vec3 y = *yio, yy = v3(0.0, 0.0, 0.0);
  double h = *hio, t = t0, lastH = h, prev_ratio = 1.0;
  int stop = 0;
  unsigned int nstep = 0;
  const double e1 = 0.7 / 7.0, e2 = -0.4 / 7.0;
  for (;;) {
    nstep++;
    if (nstep > o->nmax) {
      *yio = y;
      *hio = h;
      return -2;
    }
    if (g_counters) {
#pragma omp atomic
      g_counters->ext_attempts++;
    }
    double endDt = tf - t;
    lastH = h;
    if (g_log_mode == 2) { /* replay: the logged accepted step */
      if (g_log_n >= g_log_cap) {
        *yio = y;
        return -9;
      }
      h = g_log[2 * g_log_n];
      stop = g_log[2 * g_log_n + 1] != 0.0;
      g_log_n++;
    } else if (o->fixedStepSize) {
      h = o->h;
    } else if (h >= endDt) {
      h = endDt;
      stop = 1;
    } else {
      lastH = h;
      stop = 0;
      if (h > o->hmax) {
        h = std_min(h, o->hmax);
      } else if (h < o->hmin) {
        *yio = y;
        *hio = h;
        return -1;
      }
    }
    or_vec3 ws, te;
    ext_stages(o, type, t, h, y, &yy, t0, p_old, v_old, &ws, &te);
    double error = std_max(vlen(te), 1.0e-16);
    double tol = o->rtol;
    double ratio = tol / error;
    double q = pow(ratio, e1) * pow(prev_ratio, e2);
    q = std_min(q, 4.0);
    if ((q > 0.81 && error < 2 * tol) || o->fixedStepSize || g_log_mode == 2) {
      if (g_log_mode == 1 && g_log_n < g_log_cap) {
        g_log[2 * g_log_n] = h;
        g_log[2 * g_log_n + 1] = stop ? 1.0 : 0.0;
        g_log_n++;
      }
      y = ws;
      t += h;
      if (stop) {
        *yio = y;
        *hio = lastH;
        return 0;
      }
    } else {
      if (stop) stop = 0;
    }
    if (!o->fixedStepSize) h = h * q;
    prev_ratio = ratio;
  }
}

/* ------------------------------------------------------------ trajectory */
/* calc_next_collision_time (src/particle.cpp:121-257) */
static void next_collision(const or_options *o, double t, double tf, or_vec3 v, or_vec3 pos, double *next_gas,
                           double *dt, char *coll_type, uint64_t *n_bounce, uint64_t *n_coll, int *finished,
                           char *wall_hit, or_rng *rng) {
  double dx, dy, dz, dtx, dty, dtz;
  if (o->gravity) {
    dx = sgn1(v.x) * o->L.x / 2.0 - pos.x;
    dz = sgn1(v.z) * o->L.z / 2.0 - pos.z;
    dtx = dx / v.x;
    dtz = dz / v.z;
    double y2 = v.y * v.y;
    if (sgn1(v.y) <= 0.0) { /* falling: time to the floor */
      dy = pos.y + o->L.y * 0.5;
      double sq = sqrt(-2.0 * OR_G * dy + y2);
      double r1 = -(sq + v.y) / OR_G;
      double r2 = (sq - v.y) / OR_G;
      dty = std_min(fabs(r1), fabs(r2));
    } else {
      double top = -0.5 * y2 / OR_G + pos.y;
      if (top < 0.5 * o->L.y) { /* apex below the ceiling: up, then down to the floor */
        double t1 = -v.y / OR_G;
        double apex = pos.y + v.y * t1 + 0.5 * OR_G * t1 * t1;
        double t2 = sqrt((-0.5 * o->L.y - apex) * 2.0 / OR_G);
        dty = t1 + t2;
      } else { /* reaches the ceiling */
        double sq = sqrt(y2 - 2.0 * OR_G * (pos.y - (0.5 * o->L.y)));
        double r1 = (-v.y + sq) / OR_G;
        double r2 = (-v.y - sq) / OR_G;
        dty = std_min(fabs(r1), fabs(r2));
      }
    }
    /* only the first offending axis is replaced */
    if (dtx < 1e-16 || isnan(dtx))
      dtx = 1e6;
    else if (dty < 1e-16 || isnan(dty))
      dty = 1e6;
    else if (dtz < 1e-16 || isnan(dtz))
      dtz = 1e6;
  } else {
    dx = sgn1(v.x) * o->L.x / 2.0 - pos.x;
    dy = sgn1(v.y) * o->L.y / 2.0 - pos.y;
    dz = sgn1(v.z) * o->L.z / 2.0 - pos.z;
    dtx = dx / v.x;
    dty = dy / v.y;
    dtz = dz / v.z;
    if (dtx < 1e-16)
      dtx = 1e6;
    else if (dty < 1e-16)
      dty = 1e6;
    else if (dtz < 1e-16)
      dtz = 1e6;
  }
  double tb = NAN; /* the reference leaves this unset when no branch matches (NaN inputs) */
  if (dtx < dty && dtx < dtz) {
    tb = dtx;
    *wall_hit = 'x';
  } else if (dty < dtx && dty < dtz) {
    tb = dty;
    *wall_hit = 'y';
  } else if (dtz < dtx && dtz < dty) {
    tb = dtz;
    *wall_hit = 'z';
  } else if (dtx == dty && dtx == dtz) {
    tb = dtx;
    *wall_hit = 'a'; /* corner */
  } else if (dtx == dty) {
    tb = dtx;
    *wall_hit = 'b'; /* x-y edge */
  } else if (dtx == dtz) {
    tb = dtx;
    *wall_hit = 'c'; /* x-z edge */
  } else if (dty == dtz) {
    tb = dty;
    *wall_hit = 'd'; /* y-z edge */
  }
  double to_gas = *next_gas - t;
  int gas_next;
  double to_col;
  if (to_gas < tb) {
    gas_next = 1;
    to_col = to_gas;
  } else if (to_gas == tb) { /* tie: the wall wins, the gas clock is redrawn */
    *next_gas += or_exponential(rng, o->tc);
    to_col = to_gas;
    gas_next = 0;
  } else {
    gas_next = 0;
    to_col = tb;
  }
  int window_end;
  double to_free;
  if (tf - t <= o->maxPosStep) {
    window_end = 1;
    to_free = tf - t;
  } else {
    window_end = 0;
    to_free = o->maxPosStep;
  }
  if (to_col <= to_free) {
    *dt = to_col;
    if (gas_next) {
      *coll_type = 'G';
      *n_coll += 1;
      *next_gas += or_exponential(rng, o->tc);
    } else {
      *n_bounce += 1;
      *coll_type = 'W';
    }
    if (to_col == to_free && window_end) *finished = 1;
  } else {
    *coll_type = 'N';
    *dt = to_free;
    if (window_end) *finished = 1;
  }
}

static void flip_specular(char wh, or_vec3 *v) {
  switch (wh) {
    case 'x': v->x *= -1.0; break;
    case 'y': v->y *= -1.0; break;
    case 'z': v->z *= -1.0; break;
    case 'a': v->x *= -1.0; v->y *= -1.0; v->z *= -1.0; break;
    case 'b': v->x *= -1.0; v->y *= -1.0; break;
    case 'c': v->x *= -1.0; v->z *= -1.0; break;
    case 'd': v->y *= -1.0; v->z *= -1.0; break;
    default: break;
  }
}

/* update_position_and_velocity (src/particle.cpp:263-388) */
static void advance(const or_options *o, double *t_old, double *t, double dt, or_vec3 *pos_old, or_vec3 *pos,
                    or_vec3 *v_old, or_vec3 *v, char coll_type, char wall_hit, or_rng *rng, bool *stop) {
  *v_old = *v;
  *t_old = *t;
  *t += dt;
  *pos_old = *pos;
  const or_vec3 a = o->gravity ? v3(0.0, OR_G, 0.0) : v3(0.0, 0.0, 0.0);
  *pos = vadd(vadd(*pos_old, vscale(dt, *v)), vscale(dt, vscale(dt, vscale(0.5, a))));
  *v = vadd(*v, vscale(dt, a));
  const double speed = vlen(*v);
  if (coll_type == 'W') {
    const double hx = o->L.x * 0.5, hy = o->L.y * 0.5, hz = o->L.z * 0.5;
    (void)hx; (void)hy; (void)hz;
    int sx = 0, sy = 0, sz = 0;
    switch (wall_hit) {
      case 'x': sx = 1; break;
      case 'y': sy = 1; break;
      case 'z': sz = 1; break;
      case 'a': sx = sy = sz = 1; break;
      case 'b': sx = sy = 1; break;
      case 'c': sx = sz = 1; break;
      case 'd': sy = sz = 1; break;
      default: break;
    }
    if (sx) pos->x = sgn1(pos->x) * o->L.x * 0.5;
    if (sy) pos->y = sgn1(pos->y) * o->L.y * 0.5;
    if (sz) pos->z = sgn1(pos->z) * o->L.z * 0.5;
    if (o->diffuse > FLT_MIN && or_uniform(rng) < o->diffuse) {
      /* cosine-law diffuse reflection */
      double phi = tr_acos(sqrt(or_uniform(rng)));
      double theta = or_unif02pi(rng);
      if (wall_hit == 'x') {
        v->x = -1 * sgn1(v->x) * speed * tr_cos(phi);
        v->y = -speed * tr_sin(phi) * tr_cos(theta);
        v->z = speed * tr_sin(phi) * tr_sin(theta);
      } else if (wall_hit == 'y') {
        v->x = speed * tr_sin(phi) * tr_cos(theta);
        v->y = -1 * sgn1(v->y) * speed * tr_cos(phi);
        v->z = speed * tr_sin(phi) * tr_sin(theta);
      } else if (wall_hit == 'z') {
        v->x = speed * tr_sin(phi) * tr_cos(theta);
        v->y = speed * tr_sin(phi) * tr_sin(theta);
        v->z = -1 * sgn1(v->z) * speed * tr_cos(phi);
      } else {
        *stop = true; /* diffuse hit on an edge or corner stops the particle */
      }
    } else {
      flip_specular(wall_hit, v);
    }
  } else if (coll_type == 'G') {
    if (o->dist == 'M') {
      v->x = or_maxboltz(rng, o->sqrtKT_m);
      v->y = or_maxboltz(rng, o->sqrtKT_m);
      v->z = or_maxboltz(rng, o->sqrtKT_m);
    } else if (o->dist == 'C') {
      or_vec3 d;
      d.x = or_normal(rng, 0.0, 1.0);
      d.y = or_normal(rng, 0.0, 1.0);
      d.z = or_normal(rng, 0.0, 1.0);
      double nrm = vlen(d);
      *v = vdivs(vscale(speed, d), nrm);
    }
  }
}

/* sanity_check (src/particle.cpp:412-444) */
static void sanity(const or_options *o, double t_old, double t, or_vec3 pos_old, or_vec3 pos, or_vec3 v,
                   or_vec3 v_old, bool *stop, int *fail) {
  const double tol = 1.0e-15;
  if (fabs(pos.x) > o->L.x / 2.0 + tol || fabs(pos.y) > o->L.y / 2.0 + tol || fabs(pos.z) > o->L.z / 2.0 + tol) {
    *stop = true;
    *fail = 1;
    return;
  }
  if (isinf(t_old) || isinf(t)) {
    *stop = true;
    *fail = 2;
    return;
  }
  if (isnan(pos_old.x) || isnan(pos_old.y) || isnan(pos_old.z) || isnan(pos.x) || isnan(pos.y) || isnan(pos.z)) {
    *stop = true;
    *fail = 3;
    return;
  }
  if (isnan(v.x) || isnan(v.y) || isnan(v.z) || isnan(v_old.x) || isnan(v_old.y) || isnan(v_old.z)) {
    *fail = 4;
    *stop = true;
  }
}

int or_event(const or_options *o, or_particles *p, int i, double tf) {
  int finished = 0;
  tl_part = i;
  tl_time = p->t[i];
  double dt = 0.0;
  next_collision(o, p->t[i], tf, p->v[i], p->pos[i], &p->next_gas[i], &dt, &p->coll_type[i], &p->n_bounce[i],
                 &p->n_coll[i], &finished, &p->wall_hit[i], &p->rng[i]);
  advance(o, &p->t_old[i], &p->t[i], dt, &p->pos_old[i], &p->pos[i], &p->v_old[i], &p->v[i], p->coll_type[i],
          p->wall_hit[i], &p->rng[i], &p->stop[i]);
  sanity(o, p->t_old[i], p->t[i], p->pos_old[i], p->pos[i], p->v[i], p->v_old[i], &p->stop[i], &p->fail[i]);
  return finished;
}

/* ------------------------------------------------------------ integratorType 6
 * integrateHamiltonian (src/integrator.cpp:745-785): y = q1 q2 ... q11 y per
 * step, q_r the rotation of the CFET8 exponent with row r of G taken forwards
 * (q1..q6) or row 12 - r backwards (q7..q11), the field at the Gauss-Legendre
 * nodes from a particle at rest at the origin (findCrossTerm with zero p, v). */
static int hamiltonian(const or_options *o, double t0, double tf, or_quat *y, double h) {
  const or_vec3 zero = v3(0.0, 0.0, 0.0);
  double t = t0;
  unsigned int nstep = 0;
  while (t < tf) {
    nstep++;
    if (nstep > o->nmax) return -2;
    double rest = tf - t;
    if (h >= rest) h = rest;
    or_vec3 B[5];
    for (int i = 0; i < 5; ++i) B[i] = omega(o, t + gl5_X[i] * h, t0, &zero, &zero);
    or_quat q[12];
    for (int r = 0; r < 5; ++r) q[11 - r] = rot_quat(magnus_exponent(cfet8_G[r], 1, B, 1.0), h);  /* q11..q7 */
    for (int r = 5; r >= 0; --r) q[r + 1] = rot_quat(magnus_exponent(cfet8_G[r], 0, B, 1.0), h);  /* q6..q1 */
    or_quat prod = qmul(q[1], q[2]);
    for (int r = 3; r <= 11; ++r) prod = qmul(prod, q[r]);
    *y = qmul(prod, *y);
    t += h;
  }
  return 0;
}

void or_floquet_frequencies(const or_options *o, double freq[OR_NW], double *dt) {
  const double t0 = 0.0, tf = (2 * M_PI) / o->w;
  const int n_prop = 100;
  or_quat y = {1.0, 0.0, 0.0, 0.0};
  for (int i = 0; i < n_prop; ++i) {
    double t1 = t0 + (tf - t0) * i / n_prop;
    double t2 = t0 + (tf - t0) * (i + 1) / n_prop;
    hamiltonian(o, t1, t2, &y, 1e-6);
  }
  /* qEigenval (src/quaternion.cpp:169-172) of the period's propagator */
  const double ez = -sqrt(1.0 - y.w * y.w);
  const double ea = fabs(atan2(ez, y.w)) / (tf - t0);
  const double eb = -ea;
  const double deltaE = ea - eb;
  for (int k = 0; k <= 11 / 2; ++k)
    for (int i = -1; i < 2; ++i) {
      const int index = k * 3 + i;
      if (index >= 0) freq[index] = deltaE * i + k * o->w;
    }
  *dt = (tf - t0) / n_prop;
}

static void spec_reset(or_spec *g) { memset(g, 0, sizeof(*g)); }

/* goertzel_stage_1 and goertzel_stage_2_vector (src/floquet.cpp:25-38) per
 * frequency, and covMat::add_outer (:107-110) with v = x (real), which adds
 * 2 (b x - a 0) to the diagonal's imaginary part. */
void or_spec_update(or_spec *g, const double freq[OR_NW], double dt, or_vec3 x) {
  for (int i = 0; i < OR_NW; ++i) {
    const double angle = freq[i] * dt;
    const or_vec3 ns = vsub(vadd(x, vscale(2 * cos(angle), g->s1[i])), g->s2[i]);
    g->s2[i] = g->s1[i];
    g->s1[i] = ns;
    const double angle2 = freq[i] * dt;
    const or_vec3 b = vscale(sin(angle2), g->s2[i]);
    const or_vec3 bx = v3(b.x * x.x, b.y * x.y, b.z * x.z);
    const or_vec3 ax0 = v3(0.0, 0.0, 0.0);  /* a * imag(v) with v real */
    g->imag[i] = vadd(g->imag[i], vscale(2, vsub(bx, ax0)));
  }
  g->n_samples += 1;
}

const or_spec *or_spectrum_of(const or_particles *p, int i) { return p->spec ? &p->spec[i] : NULL; }

/* integrateSpectrum (src/integrator.cpp:724-743): samples on the grid of
 * multiples of h inside (t0, tf], each the noise field findNoiseTerm (:72-80)
 * halved: gamma (v x E / c^2 + grad(p) + testNoise(t)) / 2. */
static int integrate_spectrum(const or_options *o, double t0, double tf, or_spec *g, const double freq[OR_NW],
                              double fdt, const or_vec3 *p_old, const or_vec3 *v_old, double h) {
  double t = (floor(t0 / h) + 1) * h;
  const double next_t = (floor(tf / h) + 1) * h;
  int n = 0;
  while (t < next_t - (h / 2)) {
    or_vec3 p, v;
    or_interpolate(o, t, t0, p_old, v_old, &p, &v);
    const or_vec3 G = v3(vdot(p, o->Gx), vdot(p, o->Gy), vdot(p, o->Gz));
    const or_vec3 a = o->noiseAmplitudes, w = o->noiseFrequencies;
    const or_vec3 N = v3(a.x * sin(w.x * t), a.y * sin(w.y * t), a.z * sin(w.z * t));
    const or_vec3 B = vadd(vadd(vscale(1.0 / OR_C2, vcross(v, o->E)), G), N);
    or_spec_update(g, freq, fdt, vdivs(vscale(o->gamma, B), 2));
    t += h;
    n++;
  }
  return n;
}

/* The frequencies of the running window loop (integratorType 6). */
static double g_spec_freq[OR_NW], g_spec_dt;

/* The per-particle window loop of runSimulationCPU (src/particle.cpp:722-803). */
static void run_particle(const or_options *o, or_particles *p, int i, double next_t, uint64_t *nseg) {
  double tf = next_t;
  double hcarry = p->h[i];
  int finished = 0;
  while (!finished && !p->stop[i]) {
    finished = or_event(o, p, i, tf);
    *nseg += 1;
    if (p->fail[i] == 0) {
      int res = 0;
      if (o->integratorType == 0)
        res = or_integrate_dop(o, p->t_old[i], p->t[i], &p->S[i], &p->pos_old[i], &p->v_old[i], &hcarry);
      else if (o->integratorType == 1)
        res = or_integrate_rk45(o, p->t_old[i], p->t[i], &p->S[i], &p->pos_old[i], &p->v_old[i], &hcarry);
      else if (o->integratorType >= 2 && o->integratorType <= 5)
        res = or_integrate_ext(o, p->t_old[i], p->t[i], &p->S[i], &p->pos_old[i], &p->v_old[i], &hcarry);
      else if (o->integratorType == 6 && p->spec)
        integrate_spectrum(o, p->t_old[i], p->t[i], &p->spec[i], g_spec_freq, g_spec_dt, &p->pos_old[i],
                           &p->v_old[i], hcarry);
      if (o->keepStepSize) p->h[i] = hcarry;
      if (res < 0) {
        p->stop[i] = true;
        p->fail[i] = res;
      }
    }
    if (p->stop[i]) {
      p->t[i] = NAN;
      p->pos[i] = v3(NAN, NAN, NAN);
      p->v[i] = v3(NAN, NAN, NAN);
      p->S[i] = v3(NAN, NAN, NAN);
    }
    p->n_steps[i] += 1;
  }
}

void or_run_until(const or_options *o, or_particles *p, double next_t, int nthreads) {
  uint64_t nseg = 0;
  if (o->integratorType == 6) {  /* the aggregators restart every window (src/particle.cpp:746-747) */
    if (!p->spec) p->spec = calloc(p->n > 0 ? (size_t)p->n : 1, sizeof(or_spec));
    for (int i = 0; i < p->n; ++i) spec_reset(&p->spec[i]);
    or_floquet_frequencies(o, g_spec_freq, &g_spec_dt);
  }
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 1) reduction(+ : nseg)
#endif
  for (int i = 0; i < p->n; ++i) run_particle(o, p, i, next_t, &nseg);
  if (g_counters) g_counters->segments += nseg;
}

/* ------------------------------------------------------------ format 'A'
 * BinaryLogger (src/logger.cpp:14-38): the options image, then per snapshot
 * t[N] f64, pos[N] xyz f64, v[N], S[N], failureState[N] i32, n_coll[N] u64,
 * n_bounce[N] u64, n_steps[N] u64. */
static void write_snapshot(FILE *f, const or_particles *p) {
  size_t n = (size_t)p->n;
  fwrite(p->t, sizeof(double), n, f);
  fwrite(p->pos, sizeof(or_vec3), n, f);
  fwrite(p->v, sizeof(or_vec3), n, f);
  fwrite(p->S, sizeof(or_vec3), n, f);
  fwrite(p->fail, sizeof(int), n, f);
  fwrite(p->n_coll, sizeof(uint64_t), n, f);
  fwrite(p->n_bounce, sizeof(uint64_t), n, f);
  fwrite(p->n_steps, sizeof(uint64_t), n, f);
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int or_main_analysis(const or_options *o, const char *out_path, int nthreads, double *run_seconds) {
  or_particles p;
  int n = o->numParticles > 0 ? o->numParticles : 0;
  if (or_particles_alloc(&p, n)) return -1;
  FILE *f = fopen(out_path, "wb");
  if (!f) {
    or_particles_free(&p);
    return -2;
  }
  or_init(o, &p, 0);
  fwrite(o, sizeof(or_options), 1, f);
  write_snapshot(f, &p);
  unsigned int nwin = (unsigned int)(int)floor((double)(o->tf - o->t0) / o->ioutInt);
  double total = 0.0;
  for (int i = 0; i < (int)nwin; ++i) {
    double next_t = ((double)i + 1.0) * o->ioutInt;
    double t0 = now_s();
    or_run_until(o, &p, next_t, nthreads);
    total += now_s() - t0;
    write_snapshot(f, &p);
  }
  fclose(f);
  or_particles_free(&p);
  if (run_seconds) *run_seconds = total;
  return 0;
}

double or_run_sample(const or_options *o, int first, int count, int nthreads, or_particles *out) {
  or_particles local;
  or_particles *p = out ? out : &local;
  if (!out && or_particles_alloc(&local, count)) return -1.0;
  or_init(o, p, first);
  unsigned int nwin = (unsigned int)(int)floor((double)(o->tf - o->t0) / o->ioutInt);
  double t0 = now_s();
  for (int i = 0; i < (int)nwin; ++i) or_run_until(o, p, ((double)i + 1.0) * o->ioutInt, nthreads);
  double el = now_s() - t0;
  if (!out) or_particles_free(&local);
  return el;
}
