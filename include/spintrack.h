/*
 * spintrack.h — C ABI of the GB300-native spin-tracking engine (sm_103a).
 *
 * Drop-in for the per-particle hot path of rtat-caltech/Spin-tracking: the
 * params.txt options, the particle engine (init / run to the next output time
 * / read the snapshot), the window driver, and binary output format 'A'.
 * Citations name the reference interface each entry point replaces
 * (paths relative to the reference repository root).
 *
 * Conventions: plain C types only; every call returns 0 (ST_OK) or a negative
 * ST_ERR_* code and never exits the process (the reference's gpuErrchk calls
 * exit(), include/particle.h:23-32); st_last_error() describes the most recent
 * failure of the calling thread.  A context is single-threaded: one host
 * thread, one CUDA stream, one device.
 */
#ifndef SPINTRACK_H
#define SPINTRACK_H

#include <stddef.h>
#include <stdint.h>
#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ST_OK 0
#define ST_ERR_ARG (-1)         /* bad argument or option value */
#define ST_ERR_CUDA (-2)        /* CUDA runtime error (message in st_last_error) */
#define ST_ERR_UNSUPPORTED (-3) /* option outside the implemented path (e.g. integratorType 6) */
#define ST_ERR_IO (-4)          /* file could not be opened or written */
#define ST_ERR_STATE (-5)       /* call out of order (e.g. run before init) */
#define ST_ERR_DEADLINE (-6)    /* device time budget ran out; state is saved and resumable */
#define ST_ERR_NOMEM (-7)       /* allocation failed */

typedef struct st_vec3 { double x, y, z; } st_vec3;

/* Field-for-field the reference's `struct options` (include/options.h:10-61),
 * same order, types and defaults: 440 bytes on LP64.  Its byte image is the
 * header of output format 'A' (src/logger.cpp:27-29). */
typedef struct st_options {
  st_vec3 B0, E, L, yi, Gx, Gy, Gz;
  double m, t0, tf, rtol, atol, beta, uround, safe, fac1, fac2, hmax, hmin, h, T;
  double sqrtKT_m, tc, gamma, V, a, w, swapStepSize, maxPosStep, ioutInt, diffuse;
  unsigned int nmax, seed;
  int integratorType, numParticles, numPerGPUBlock, iout;
  char dist;
  bool gas_coll, gravity, fixedStepSize, keepStepSize;
  st_vec3 noiseAmplitudes, noiseFrequencies;
} st_options;

/* Host (or device) arrays of numParticles entries each, one per snapshot field
 * of format 'A' (src/logger.cpp:14-25).  A NULL member is skipped. */
typedef struct st_state_view {
  double *t;
  st_vec3 *pos, *v, *S;
  int32_t *fail;
  uint64_t *n_coll, *n_bounce, *n_steps;
} st_state_view;

/* Device-resident particle state, structure of arrays (borrowed pointers,
 * valid until st_destroy).  Component arrays of length n_total. */
typedef struct st_device_soa {
  int64_t n_total;
  double *t, *pos_x, *pos_y, *pos_z, *v_x, *v_y, *v_z, *S_x, *S_y, *S_z, *h, *next_gas;
  int32_t *fail;
  uint64_t *n_coll, *n_bounce, *n_steps;
  uint8_t *stop;
} st_device_soa;

/* Which kernel advances the particles. */
#define ST_KERNEL_PLAIN 0      /* one thread per particle, one launch per output window */
#define ST_KERNEL_PERSISTENT 1 /* persistent work-queue kernel, lanes refilled as particles finish */

/* Launch configuration of the persistent kernel (autotuned when zero). */
typedef struct st_launch_config {
  int block_threads;   /* threads per block; 0 = autotune */
  int blocks_per_sm;   /* resident blocks per SM; 0 = autotune */
  int variant;         /* kernel variant index (register budget); -1 = autotune */
} st_launch_config;

/* ---- library ---------------------------------------------------------- */
int st_version(void);
const char *st_last_error(void);

/* ---- options (include/options.h, src/optionsParser.cpp) ---------------- */
size_t st_options_size(void);
/* options{} default member values, include/options.h:10-61 */
void st_options_default(st_options *opt);
/* parseLine, src/optionsParser.cpp:40-175.  Returns 0 when the key was
 * applied, 1 for an unrecognised key (ignored, as the reference does),
 * ST_ERR_ARG for a line with fewer than two fields or a malformed number. */
int st_parse_line(st_options *opt, const char *line);
/* optionParser, src/optionsParser.cpp:177-197: defaults, then every line of
 * the file.  A missing file leaves the defaults (as the reference does) and
 * returns ST_ERR_IO so the caller can tell. */
int st_parse_params(const char *path, st_options *opt);
/* Derived parameters of mainAnalysis, src/simulation.cpp:9-11:
 * tc = 1.6e-4 m / (k T^8), sqrtKT_m = sqrt(k T / m). */
void st_derive(st_options *opt);
/* Number of output windows of a run: floor((tf - t0) / ioutInt),
 * src/simulation.cpp:43. */
int st_num_windows(const st_options *opt);

/* ---- engine: class particle (include/particle.h:87-314) --------------- */
typedef struct st_ctx st_ctx;
/* particle::particle(options), include/particle.h:90-166: allocates the
 * device state for opt->numParticles particles (taken as given: call
 * st_derive first, as mainAnalysis does). */
int st_create(const st_options *opt, int device, st_ctx **out);
/* Batched form: nsets parameter sets, set s holding sets[s].numParticles
 * particles seeded exactly as an independent reference run with sets[s]. */
int st_create_batch(const st_options *sets, int nsets, int device, st_ctx **out);
/* particle::~particle, include/particle.h:167-240 */
void st_destroy(st_ctx *ctx);
/* particle::initParticles, include/particle.h:241-252 (initParticlesCPU
 * semantics, src/particle.cpp:638-710). */
int st_init(st_ctx *ctx);
/* particle::runSimulation(nextTOut), src/particle.cpp:865-876: advance every
 * particle to next_t with the plain kernel (one launch). */
int st_run_until(st_ctx *ctx, double next_t);
/* Window loop of mainAnalysis, src/simulation.cpp:43-61: advance windows
 * [w_begin, w_end) (window i ends at (i+1)*ioutInt), clamped per set to its
 * own window count.  If snap != NULL, the state at the end of each window is
 * written to it: (w_end - w_begin) consecutive blocks, each laid out as
 * st_snapshot_bytes(ctx) bytes (see st_snapshot_field_offset).  snap is a
 * device pointer. */
int st_run_windows(st_ctx *ctx, int kernel, int w_begin, int w_end, void *snap);
/* Bytes of one device snapshot block and the offset of field f within it
 * (f: 0 t, 1 pos_x, 2 pos_y, 3 pos_z, 4 v_x, 5 v_y, 6 v_z, 7 S_x, 8 S_y,
 * 9 S_z, 10 fail(i32), 11 n_coll, 12 n_bounce, 13 n_steps, 14 precession
 * turns (i32, see st_gather_phase); each field an array over all particles,
 * 256-byte aligned). */
size_t st_snapshot_bytes(const st_ctx *ctx);
size_t st_snapshot_field_offset(const st_ctx *ctx, int field);
/* particle::outputData, src/particle.cpp:852-862: synchronise and copy the
 * eight snapshot fields of every particle to host arrays. */
int st_read_state(st_ctx *ctx, const st_state_view *host);
/* Copy every particle's spin into a dense device array (3 doubles per
 * particle, set order) and wait for the copy. */
int st_gather_spins(st_ctx *ctx, double *dst_device);
/* Borrowed device pointers to the SoA state. */
int st_device_state(st_ctx *ctx, st_device_soa *out);
int st_synchronize(st_ctx *ctx);
/* The context's CUDA stream (cudaStream_t), for callers that order their own
 * work or time kernels with events on it. */
void *st_get_stream(st_ctx *ctx);
/* Replace every set's parameters (same particle counts) without reallocating:
 * the device parameter table is re-uploaded; call st_init to restart.  Used
 * for parameter scans.  When gas collisions or an integrator type change, an
 * autotuned launch configuration (or a chosen one that has no kernel for the
 * new types) is dropped and tuned again at the next run.  No counterpart in the reference, which takes options
 * only at construction (include/particle.h:90). */
int st_set_params(st_ctx *ctx, const st_options *sets, int nsets);
/* Bytes of the device parameter table that st_set_params uploads. */
size_t st_param_table_bytes(const st_ctx *ctx);
/* Persistent-kernel launch configuration (NULL = autotune on first use). */
int st_set_launch_config(st_ctx *ctx, const st_launch_config *cfg);
int st_get_launch_config(const st_ctx *ctx, st_launch_config *cfg);
/* Number of persistent-kernel variants (valid st_launch_config.variant
 * values are 0 .. count-1) and the name of one, for external tuners.  The
 * autotuner offers the flattened ("flat_*") and trajectory-ahead ("ahead_*")
 * variants; the warp-specialised ("split_*") and three-lanes-per-particle
 * ("tpp3_*") ones run only when chosen here. */
int st_launch_variant_count(void);
const char *st_launch_variant_name(int variant);
/* Device time budget for each following run call, in seconds (0 = none).
 * When it runs out, kernels save the particle state and the call returns
 * ST_ERR_DEADLINE; calling again resumes. */
int st_set_deadline(st_ctx *ctx, double seconds);
/* Work counters of the last run call: DOP853, RK45 and integratorType 2-5
 * step attempts, trajectory segments, and kernels launched.  st_run_windows enqueues its
 * launches as one CUDA graph, captured on the first call with a given
 * (kernel, window range, snapshot buffer, launch configuration, deadline) and
 * replayed by later calls: graph_launches = 1 for such a call, graph_captures
 * = 1 when it captured a new graph. */
typedef struct st_counters {
  uint64_t dop_attempts, rk45_attempts, segments, kernel_launches;
  uint64_t graph_launches, graph_captures;
  uint64_t ext_attempts;  /* step attempts of integratorType 2-5 */
} st_counters;
int st_get_counters(const st_ctx *ctx, st_counters *out);

/* Allocation-free run, for callers that cannot allocate device memory when
 * they run the tracker (a host whose memory pool owns the GPU, or a hot path
 * that must not call cudaMalloc/cudaFree because they synchronise the device).
 * No counterpart in the reference.  Equivalent to st_create_batch + st_init +
 * st_run_windows(ST_KERNEL_PERSISTENT, 0, w_end) on the current device and
 * the caller's stream, but every byte it touches is either the caller's
 * `state` buffer or a 8 KiB scratch array compiled into the library (work
 * queue cursor, counters, parameter table), held by each GPU that loads the
 * library until the process exits.  It calls no cudaMalloc/cudaFree.
 *   state == NULL: writes the required buffer size to *state_bytes, returns.
 *   state != NULL: a 256-byte aligned device buffer of *state_bytes bytes;
 *     on return it holds the particle state after window w_end as 28 arrays
 *     over all particles (sets in order), each starting on a 256-byte
 *     boundary: t, pos_x, pos_y, pos_z, v_x, v_y, v_z, S_x, S_y, S_z (f64),
 *     fail (i32), n_coll, n_bounce, n_steps (u64), then internal fields.
 * At most 8 parameter sets per call (ST_ERR_ARG beyond).  Every call shares
 * the scratch and it keeps the last call's contents; each call clears what
 * must start at zero, so calls that overlap on the GPU race and must not be
 * issued.  The first call on a device (and the first after its context was
 * reset) looks the scratch address up with cudaGetSymbolAddress; make it
 * before any stream capture.  The launch is fixed (the flattened persistent
 * kernel, 128-thread blocks, as many per SM as fit; no autotuner, no
 * type-grouped work order): same results as st_run_windows, possibly lower
 * throughput.  Returns ST_ERR_CUDA when a lane reports that it could not make
 * progress, as st_run_windows does.  Synchronises `stream` (a cudaStream_t,
 * NULL = default stream) before returning. */
int st_run_noalloc(const st_options *sets, int nsets, void *state, size_t *state_bytes, int w_end, void *stream);

/* ---- discrete adjoint (DOP853 or Magnus CFET8, fixed accepted steps) --- */
/* Gradient parameters, in this order: the gradient tensor rows Gx, Gy, Gz
 * (9: B_i = dot(pos, G_i)), B0 (3), E (3), pulse amplitude a and angular
 * frequency w (2). */
#define ST_NUM_THETA 17
/* Forward pass for st_adjoint_backward, from a freshly initialised context
 * (st_init): advances every particle through windows [0, w_end) exactly as
 * st_run_windows does (the trajectory-ahead kernel), and writes the adjoint's
 * tape: every accepted step (y, x, h) and every integrated segment
 * (t0, p0, v0) of every particle, in pages of a device pool of tape_bytes
 * (0 = up to 85% of free device memory).  It also keeps a full-state
 * checkpoint every windows_per_checkpoint windows (0 = chosen so the
 * checkpoints take at most 10% of free memory).  A run of four or more
 * checkpoint intervals is recorded in pieces: the first interval's tape
 * projects the whole tape; when that does not fit the pool, only the last
 * intervals that fit are stored (the rest of the run keeps checkpoints only)
 * and st_adjoint_backward takes them first, then replays window chunks of the
 * earlier intervals from the checkpoints (and, if one window's tape does not
 * fit, groups of particles), so results do not depend on the pool size.  All sets of the context integrate with
 * DOP853 (integratorType 0) or all with Magnus CFET8 (2); the linear grad
 * hook only.
 * No counterpart in the reference (it has no derivatives). */
int st_adjoint_record(st_ctx *ctx, int w_end, size_t tape_bytes, int windows_per_checkpoint);
/* Backward pass: given dL/dS_final for every particle (device array,
 * 3 doubles per particle, set order), writes dL/dtheta per particle (device
 * array, ST_NUM_THETA doubles per particle); sum over a set's particles for
 * the set's gradient.  Particles that stopped (failure codes) get zeros.
 * flags bit 0: also differentiate the pulse (a, w), one sincos per stage. */
int st_adjoint_backward(st_ctx *ctx, const double *dL_dS, double *grad, int flags);
/* The backward for nloss losses at once: dL_dS holds nloss blocks of
 * 3 doubles per particle, grad receives nloss blocks of ST_NUM_THETA doubles
 * per particle.  When the tape did not fit, each chunk of the run is replayed
 * once for all the losses.  No counterpart in the reference. */
int st_adjoint_backward_multi(st_ctx *ctx, int nloss, const double *dL_dS, double *grad, int flags);
/* What the last record / backward pair did (no reference counterpart). */
typedef struct {
  uint64_t tape_bytes_used;   /* tape written by the record pass (all of it, stored or not) */
  uint64_t tape_bytes_pool;   /* size of the tape pool */
  int32_t resident;           /* 1: the record pass's tape fitted, the backward needs no replay */
  int32_t checkpoints;        /* state checkpoints kept by the record pass */
  int32_t windows_per_checkpoint;
  int32_t replays;            /* replay launches of the last backward */
  int32_t groups;             /* particle-group replays among them */
  int32_t tail_from;          /* when the whole tape did not fit: the checkpoint interval from which the record
                                 pass kept it (the backward replays only the intervals before); = checkpoints
                                 when nothing was kept apart */
  int32_t record_launches;    /* kernel launches of the record pass */
  int32_t pad;
} st_adjoint_stats;
int st_adjoint_get_stats(const st_ctx *ctx, st_adjoint_stats *out);

/* Unwrapped precession phase of every particle about x, accumulated on the
 * device over the whole run: atan2(Sz, Sy) + 2 pi * turns, where turns counts
 * the accepted steps that carried the spin's (y, z) projection across the
 * cut at +-pi (Sz changing sign with Sy < 0; a step at rtol 1e-12 turns the
 * spin by far less than pi).  Unlike phases taken from snapshots, it stays
 * continuous however long the window.  dst: device array, one double per
 * particle.  No counterpart in the reference (its scripts wrap phases). */
int st_gather_phase(st_ctx *ctx, double *dst);

/* ---- ensemble statistics (on the device) ------------------------------ */
/* The reference computes these in its analysis scripts from the output file
 * (scripts/nedmSim.py:151-179 shiftDatapoints,
 * benchmarks/CheckingFrequencyShiftFromEField.ipynb analyzeDataset); here
 * they are reduced on the device, so a parameter sweep needs no file.  Over
 * the particles of one set with failureState 0 and a finite phase
 * phi = atan2(Sz, Sy): the phases are aligned to the most populated of 1000
 * equal bins (numpy.histogram binning) and clipped at 5 standard deviations,
 * as shiftDatapoints does; frequency shift = wrap(phase_mean - phase_expected)
 * / (2 pi t) with phase_expected = atan2(cos(w t), sin(w t)),
 * w = gamma |B0| sign(B0x).  phase_stderr = phase_std / sqrt(n_phase) (the
 * notebook divides by the square root of the number of snapshots instead). */
typedef struct {
  double t;               /* time of the snapshot (first counted particle) */
  int64_t n_valid;        /* particles counted */
  int64_t n_phase;        /* of those, kept by the 5-sigma clip */
  double mean_S[3];       /* mean spin of the counted particles */
  double polarisation;    /* |mean_S| */
  double phase_mean;      /* aligned, clipped mean phase, wrapped to [-pi, pi] */
  double phase_std;       /* population standard deviation of the same phases */
  double phase_stderr;    /* phase_std / sqrt(n_phase) */
  double phase_expected;
  double freq_shift;      /* Hz */
  double freq_shift_err;  /* phase_stderr / (2 pi t), Hz */
  /* the unwrapped phase (st_gather_phase) over the counted particles: mean,
   * population std, and its shift against the continuous expected phase
   * phi0 - w t (phi0 = atan2(yi_z, yi_y)), in Hz: no +-pi ambiguity */
  double phase_unwrapped_mean;
  double phase_unwrapped_std;
  double freq_shift_unwrapped;
} st_ensemble;
/* snap: a device snapshot block (st_snapshot_bytes) or NULL for the current
 * state; set: parameter-set index. */
int st_ensemble_stats(st_ctx *ctx, const void *snap, int set, st_ensemble *out);

/* FP64 FMA issue-rate probe (TFLOP/s, FMA = 2 flops): eight independent
 * DFMA chains per thread on every SM.  No counterpart in the reference; it is
 * the roofline denominator for the step kernels, which are FP64-pipe bound. */
int st_probe_fp64_peak(int device, double *tflops);
/* The trajectory's correctly rounded libm replacements (log, sin, cos, acos;
 * their results equal the host C library's wherever those are correctly
 * rounded), evaluated over n doubles of a device array x into device array y
 * on the current device, synchronously: fn 0 log, 1 sin, 2 cos, 3 acos,
 * 4 and 5 sin and cos of acos(x) as a cosine-law reflection takes them;
 * fn 8-11: the accurate evaluations of log, sin, cos and acos alone (the
 * fallback the others take when a fast result's rounding is uncertain).
 * For tests; no reference counterpart. */
int st_crmath_eval(int fn, const double *x, double *y, int64_t n);

/* ---- integratorType 6: the noise spectrum ------------------------------- */
/* A context whose sets all have integratorType 6 integrates no spin: along
 * every segment it samples the noise field gamma (v x E / c^2 + grad(p) +
 * testNoise(t)) / 2 on the grid of multiples of h and runs 17 Goertzel
 * recursions per particle, at the Floquet frequencies of the dressed spin
 * (integrateSpectrum and SpectrumAggregator, src/integrator.cpp:724-743,
 * src/floquet.cpp:25-156); the aggregators restart at every window, as the
 * reference's window loop resets them (src/particle.cpp:746-747).  Type 6 sets
 * need w != 0 and cannot share a context with types 0-5; both kernel
 * selectors run the spectrum kernel. */
#define ST_SPECTRUM_FREQS 17
/* floquet_diagonalize (src/integrator.cpp:824-867): the 17 Goertzel
 * frequencies (rad/s) and the Goertzel step dt of opt's dressing field. */
int st_floquet_frequencies(const st_options *opt, double *freq, double *dt);
/* Every particle's aggregator after the last window: host arrays of
 * numParticles x 17 x 3 doubles (s1, s2: the recursion's last two values;
 * imag: the Laplace term of the covariance diagonal, covMat::imag_diag) and
 * the samples taken.  The reference keeps them in SpectrumAggregator
 * (include/floquet.h:76-95, particle::getSpectrumAggregators). */
int st_spectrum_state(st_ctx *ctx, double *s1, double *s2, double *imag, int64_t *n_samples);
/* The covariance spectrum of a set summed over its particles in index order:
 * variance[k][r][q] (complex, 17 x 3 x 3 x {re, im}) = sum over particles of
 * c_r conj(c_q) with c = s1 - cos(w_k dt) s2 + i sin(w_k dt) s2, minus i imag
 * on the diagonal (goertzel_stage_2 and get_covariance_spectrum,
 * src/floquet.cpp:40-47, 130-145; CovarianceSpectrum::add, :74-79).  The
 * reference's own reduction nests its tree loops the wrong way round
 * (src/particle.cpp:826-834) and its GPU path does not reduce; this is the
 * plain sum they aim at, unnormalised, with the samples in *n_samples. */
int st_covariance_spectrum(st_ctx *ctx, int set, double *variance, int64_t *n_samples);

/* ---- driver: mainAnalysis (src/simulation.cpp:8-96) -------------------- */
/* Derive tc/sqrtKT_m, create, init, write the options header and the t0
 * snapshot, run every window with `kernel`, append a snapshot per window
 * (format 'A', src/logger.cpp:14-38).  run_seconds (may be NULL) receives the
 * wall time of the window loop excluding file writes.  A path ending in .h5 or
 * .hdf5 (any case) is refused with ST_ERR_UNSUPPORTED, as by a reference
 * build without HDF5 (createLogger, src/logger.cpp:192-204). */
int st_main_analysis(const st_options *opt, const char *out_path, int device, int kernel, double *run_seconds);
/* Format 'A' writer pieces, for callers that hold their own state. */
int st_write_header(void *file /* FILE* */, const st_options *opt);
int st_write_snapshot(void *file /* FILE* */, int n, const st_state_view *host);

#ifdef __cplusplus
}
#endif
#endif
