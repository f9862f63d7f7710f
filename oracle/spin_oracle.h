/*
 * ORACLE — test infrastructure only.  A plain-C restatement of the reference
 * Spin-tracking hot path (rtat-caltech/Spin-tracking), used by tests/ as the
 * parity checker and by bench.py as the timed CPU baseline.  The product
 * (spin-tracking_gb300/) never links, loads or calls anything here.
 *
 * Every floating-point expression keeps the reference's evaluation order so
 * that, compiled with -ffp-contract=off, results are bit-identical to the
 * reference CPU build on the same host (checked against golden vectors made by
 * the reference itself, tests/golden/).
 */
#ifndef SPIN_ORACLE_H
#define SPIN_ORACLE_H

#include <stdint.h>
#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { double x, y, z; } or_vec3;

/* Field-for-field image of the reference's `struct options`
 * (include/options.h:10-61): 440 bytes on LP64, also the format-'A' header. */
typedef struct {
  or_vec3 B0, E, L, yi, Gx, Gy, Gz;
  double m, t0, tf, rtol, atol, beta, uround, safe, fac1, fac2, hmax, hmin, h, T;
  double sqrtKT_m, tc, gamma, V, a, w, swapStepSize, maxPosStep, ioutInt, diffuse;
  unsigned int nmax, seed;
  int integratorType, numParticles, numPerGPUBlock, iout;
  char dist;
  bool gas_coll, gravity, fixedStepSize, keepStepSize;
  or_vec3 noiseAmplitudes, noiseFrequencies;
} or_options;

/* Reference rngState (include/particle.h:52-59). */
typedef struct {
  uint64_t x, y, z, w;
  double spare;
  bool has_spare;
} or_rng;

/* Per-particle state, structure of arrays, owned by the caller. */
typedef struct {
  int n;
  or_vec3 *S, *v, *v_old, *pos, *pos_old;
  double *t, *t_old, *h, *next_gas;
  or_rng *rng;
  int *fail;
  uint64_t *n_bounce, *n_coll, *n_steps;
  bool *stop;
  char *coll_type, *wall_hit;
  struct or_spec *spec;  /* integratorType 6: one noise-spectrum aggregator per particle (allocated by or_init) */
} or_particles;

/* Noise-spectrum aggregator of integratorType 6 (SpectrumAggregator,
 * include/floquet.h:76-95): per Goertzel frequency, the recursion's last two
 * values s1, s2 and the Laplace term of the covariance diagonal (covMat
 * imag_diag; its other members stay zero), and the samples taken. */
#define OR_NW 17
typedef struct or_spec {
  or_vec3 s1[OR_NW], s2[OR_NW], imag[OR_NW];
  int64_t n_samples;
} or_spec;

size_t or_options_size(void);
void or_options_default(or_options *opt);
/* parseLine (src/optionsParser.cpp:40-175); returns 0 if the key was used. */
int or_parse_line(or_options *opt, const char *line);
/* optionParser (src/optionsParser.cpp:177-197); missing file = defaults. */
int or_parse_file(const char *path, or_options *opt);
/* tc and sqrtKT_m as mainAnalysis derives them (src/simulation.cpp:9-11). */
void or_derive(or_options *opt);

/* RNG (src/particle.cpp:33-119). */
void or_rng_seed(or_rng *r, unsigned int seed, unsigned int ipart);
uint64_t or_xoshiro(or_rng *r);
double or_uniform(or_rng *r);
double or_normal(or_rng *r, double mean, double std);
double or_exponential(or_rng *r, double tc);

/* Particle engine (src/particle.cpp:638-825). */
int or_particles_alloc(or_particles *p, int n);
void or_particles_free(or_particles *p);
void or_init(const or_options *opt, or_particles *p, int first_index);
void or_run_until(const or_options *opt, or_particles *p, double next_t, int nthreads);

/* Steppers over one ballistic segment (src/integrator.cpp:90-337). */
int or_integrate_dop(const or_options *opt, double t0, double tf, or_vec3 *y, const or_vec3 *p_old,
                     const or_vec3 *v_old, double *h);
int or_integrate_rk45(const or_options *opt, double t0, double tf, or_vec3 *y, const or_vec3 *p_old,
                      const or_vec3 *v_old, double *h);
/* integratorType 2-5 (src/integrator.cpp:339-722): Magnus CFET8, RK45 with
 * quaternions, RKF45, RKF45 with quaternions; the type is opt->integratorType. */
int or_integrate_ext(const or_options *opt, double t0, double tf, or_vec3 *y, const or_vec3 *p_old,
                     const or_vec3 *v_old, double *h);

/* Ballistic interpolation (src/integrator.cpp:48-61). */
void or_interpolate(const or_options *opt, double t, double t0, const or_vec3 *p_old, const or_vec3 *v_old,
                    or_vec3 *p_out, or_vec3 *v_out);

/* One segment event: calc_next_collision_time + update_position_and_velocity
 * + sanity_check (src/particle.cpp:121-444) for particle i with window end tf.
 * Returns the `finished` flag. */
int or_event(const or_options *opt, or_particles *p, int i, double tf);

/* mainAnalysis (src/simulation.cpp:8-96) writing format 'A' to out_path.
 * opt is taken as given (call or_derive first, as the reference does).
 * Returns 0 on success; *run_seconds receives the summed window time. */
int or_main_analysis(const or_options *opt, const char *out_path, int nthreads, double *run_seconds);

/* Bounded CPU baseline: particles [first, first+count) of opt's run, all
 * windows, no file output.  Returns the wall seconds spent. */
double or_run_sample(const or_options *opt, int first, int count, int nthreads, or_particles *out);

/* Instrumented count of DOP853 step attempts and segments, for the roofline
 * work model: filled by or_run_until when non-null. */
typedef struct { uint64_t dop_attempts, rk45_attempts, segments, ext_attempts; } or_counters;
void or_set_counters(or_counters *c);

/* Frozen accepted-step log for finite-difference checks: mode 1 records every
 * accepted DOP853 / type 2-5 step as (h, last), mode 2 replays the record in place of the
 * step controller, 0 = off.  Single-threaded runs only. */
void or_set_step_log(double *buf, int64_t cap, int mode);
int64_t or_step_log_count(void);

/* The trajectory's elementary functions (log, acos, sin, cos): mode 0 the
 * host C library (the reference's results, default), 1 correctly rounded
 * (binary128 evaluation, one rounding), 2 the host library, 3 correctly
 * rounded but for the k-th call per particle whose host result differs
 * (k from or_set_math_pick; -1 none), which takes the host result.  In modes
 * 1-3 the audit arrays (n local particle slots, zeroed by the caller) receive
 * per particle the number of calls whose two results differ and, for the
 * first (mode 3: the picked one), the particle time at the start of its
 * segment, the function (OR_FN_*) and the argument; null arrays turn the
 * audit off. */
/* floquet_diagonalize (src/integrator.cpp:824-867): the 17 Goertzel
 * frequencies and the step dt of the dressed-spin Floquet analysis, from the
 * one-period propagator of the field gamma (B0 + pulse) (integrateHamiltonian,
 * src/integrator.cpp:745-785, 100 intervals of 1e-6 s Magnus CFET8 steps). */
void or_floquet_frequencies(const or_options *opt, double freq[OR_NW], double *dt);
/* SpectrumAggregator::update (src/floquet.cpp:113-120) with the sample x. */
void or_spec_update(or_spec *g, const double freq[OR_NW], double dt, or_vec3 x);
/* The aggregator of local particle slot i (after or_run_until). */
const or_spec *or_spectrum_of(const or_particles *p, int i);

enum { OR_FN_LOG = 0, OR_FN_SIN = 1, OR_FN_COS = 2, OR_FN_ACOS = 3 };
void or_set_math_mode(int mode);
void or_set_math_pick(const int64_t *k);
void or_set_math_audit(int64_t *count, double *first_t, int *first_fn, double *first_arg, int n);
/* y[k] = fn(x[k]) with the host library (mode 0) or correctly rounded (mode 1). */
void or_math_eval(int fn, int mode, const double *x, double *y, int64_t n, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
