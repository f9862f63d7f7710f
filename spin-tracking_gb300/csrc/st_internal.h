// Internal types shared by the host library (st_api.cpp) and the kernels
// (st_kernels.cu).  Not part of the public ABI (include/spintrack.h).
#pragma once

#include <stdint.h>
#include "spintrack.h"

namespace st {

// Trajectory / integrator constants of the reference (include/options.h:7-8).
constexpr double kGravity = -9.81;
constexpr double kC2 = 299792458.0 * 299792458.0;

// One parameter set, laid out for the device.  Derived once on the host from
// an st_options; every kernel reads it through a pointer into a device table
// (broadcast loads for a single-set run, per-lane loads in batched runs).
struct SetParams {
  // ---- trajectory (src/particle.cpp:121-444)
  double Lx, Ly, Lz;              // box edges
  double maxPosStep, tc, sqrtKT_m, diffuse, V;
  // ---- spin field (src/integrator.cpp:40-88)
  double gamma;
  double B0x, B0y, B0z, Ex, Ey, Ez;
  double Gx[3], Gy[3], Gz[3];     // rows: B_i = dot(pos, G_i)
  double a, w;                    // pulse amplitude and angular frequency
  double inv_c2;                  // 1.0 / c^2 as the reference evaluates it
  // Field constants of the segment polynomial, filled on the device from the
  // st_grad hook by launch_prepare_sets:
  //   Omega(tau) = o0 + tau (o1 + tau o2),
  //   o0 = gB0 + sum_j p0_j gGc[j] + v0 x gEc,  o1 = sum_j v0_j gGc[j] + o1g,  o2 = o2c.
  double gB0[3];                  // gamma * B0
  double gGc[3][3];               // gamma * grad(e_j): column j of the gradient tensor
  double gEc[3];                  // gamma * E / c^2
  double o1g[3];                  // gamma * (g yhat x E) / c^2 (gravity)
  double o2c[3];                  // gamma * (g / 2) * grad(yhat) (gravity)
  // ---- stepper (src/integrator.cpp:90-337)
  double rtol, atol, hmin, hmax, h0, safe, fac1, fac2, beta;
  double facc1, facc2, expo1, inv_safe;
  // ---- windows (src/simulation.cpp:43-49)
  double t0, tf, ioutInt;
  double yi_x, yi_y, yi_z;
  unsigned int nmax, seed;
  int integrator;                 // 0 DOP853, 1 RK45, 2 Magnus CFET8, 3 RK45 with quaternions,
                                  // 4 RKF45, 5 RKF45 with quaternions; other values: trajectory only
  int nwin;                       // floor((tf - t0) / ioutInt)
  int gravity, gas, fixed, keep;
  int dist;                       // 'C' or 'M'
  int64_t first;                  // global index of the set's first particle
  int64_t n;                      // particles in the set
};

// Device SoA particle state.  RNG state and bookkeeping live beside the
// physical state so a particle can be resumed from memory at any window end.
struct DeviceState {
  int64_t n;
  double *t, *px, *py, *pz, *vx, *vy, *vz, *Sx, *Sy, *Sz, *h, *next_gas;
  uint64_t *rx, *ry, *rz, *rw;    // xoshiro words
  double *rspare;                 // cached second normal
  uint8_t *rhas;                  // spare valid
  int32_t *fail;
  uint64_t *n_coll, *n_bounce, *n_steps;
  uint8_t *stop, *coll, *wall;
  int32_t *set;                   // parameter set of each particle
  int32_t *w_done;                // windows completed
  int32_t *turns;                 // precession turns: unwrapped phase = atan2(Sz, Sy) + 2 pi turns
};

// Snapshot block: 15 field arrays over all particles (the 14 of the state
// view, then the precession turns), each padded to 256 B.
constexpr int kSnapFields = 15;
struct SnapLayout {
  int64_t n;
  size_t off[kSnapFields];
  size_t bytes;
};

// Device-side run counters and status (one per context).
struct RunStatus {
  unsigned long long dop_attempts;
  unsigned long long rk45_attempts;
  unsigned long long segments;
  unsigned long long ext_attempts;  // step attempts of integrator types 2-5
  unsigned long long queue_head;   // persistent-kernel work queue cursor
  unsigned long long deadline_ns;  // %globaltimer value after which lanes stop (0 = none)
  int deadline_hit;
  int pad;                         // set by a kernel that detected an internal logic error
};

struct RunArgs {
  const SetParams* sets;
  int nsets;
  const int64_t* order;           // work order (persistent kernel), may be null
  int64_t nitems;                 // items of the work queue (entries of order, else particles)
  DeviceState s;
  RunStatus* status;
  char* snap;                     // snapshot buffer base (device), may be null
  SnapLayout snap_layout;
  int w_begin, w_end;             // window range of this call
  int deadline_armed;             // read RunStatus::deadline_ns at kernel start
  int count_work;                 // accumulate attempt counters
  int any_gas;                    // some set has gas collisions (else gas-free kernels may run)
  int any_ext;                    // some set integrates with type 2-5 (the EXT kernels must run)
  int any_rk45;                   // some set integrates with RK45 (type 1)
};

// Discrete adjoint (st_adjoint.cu): gradient of L(S_final) with respect to
// theta = [Gx(3), Gy(3), Gz(3), B0(3), E(3), a, w].
constexpr int kNumTheta = 17;

// The adjoint's tape, written by the trajectory-ahead kernel (k_batched with
// its tape switch on): pages of kTapePageD doubles from one pool.  Every
// particle owns two chains of pages, linked last to first: its accepted
// DOP853 steps (y, x, h) and its integrated segments (t0, p0, v0).  A step
// is the first of its segment exactly when x equals the segment's t0: the
// first accepted step starts at t0 (rejected attempts do not move x), and
// later steps cannot return there (a zero-length segment has one step).  The
// sign of h carries no flag: a segment shorter than hmin is overshot by an
// hmin step and closed by a negative one, as in the reference.
constexpr int kTapePageD = 320;
constexpr int kTapeStepD = 5, kTapeStepsPerPage = 64;
constexpr int kTapeSegD = 8, kTapeSegsPerPage = 40;
// Tape consistency report: [0] code (0 = none), [1] particle, [2..5] step page,
// step record, segment page, segment record, [6..7] steps and segments of the
// particle's tape, [8..9] steps and segments walked back when it was found.
constexpr int kTapeErrorSlots = 10;
struct TapeArgs {
  double* pool;
  int32_t* page_prev;             // per page: the chain's previous page (-1: none)
  unsigned long long* pool_head;  // page bump allocator (may run past pool_pages)
  int64_t pool_pages;
  // per particle
  int32_t *step_page, *step_fill; // last page of the step chain and its records
  int32_t *seg_page, *seg_fill;   // last page of the segment chain and its records
  int64_t *nsteps, *nsegs;        // records of each chain, counted even when not stored
  int32_t* complete;              // 1: both chains stored in full
  int append;                     // 1: continue each particle's chains from the cursors of the last close
  // state checkpoints written at window ends (record pass): state k is the
  // state after window k * ckpt_every - 1, at ckpt.<field> + k * ckpt_stride bytes
  DeviceState ckpt;
  int64_t ckpt_stride;
  int ckpt_every, ckpt_count;
  // backward pass
  double* lam;                    // per particle: dL/dS at the end of the taped span (in, out)
  double* grad;                   // per particle: kNumTheta accumulators (+=)
  const uint8_t* final_stop;      // per particle: stopped at the end of the forward run
  int pulse_grads;
  long long* error;               // kTapeErrorSlots: first inconsistency found (code, particle, cursors)
};
// The trajectory-ahead kernel with its tape switch on (st_kernels.cu).
int launch_crmath_eval(int fn, const double* x, double* y, int64_t n, void* stream);
int launch_tape_record(const RunArgs& a, const TapeArgs& t, int blocks, void* stream);  // a.any_ext: Magnus
int tape_record_block();
int tape_record_max_blocks_per_sm(int ext);
int launch_adj_backward(const RunArgs& a, const TapeArgs& t, int blocks, int magnus, void* stream);
int adj_backward_block();
int adj_backward_max_blocks_per_sm(int magnus);

// Ensemble statistics (st_ensemble.cu).
int ensemble_device(const double* t, const double* Sx, const double* Sy, const double* Sz, const int32_t* fail,
                    const int32_t* turns, int64_t first, int64_t n, double* ctl, double* part, unsigned int* hist,
                    int max_blocks, void* stream);
int ensemble_ctl_count();
constexpr int kEnsMaxBlocks = 1024, kEnsHistBins = 1000;
enum { ENS_COUNT = 0, ENS_SX, ENS_SY, ENS_SZ, ENS_MIN, ENS_MAX, ENS_T, ENS_EDGE0, ENS_EDGE1, ENS_LOC, ENS_MEAN1,
       ENS_STD1, ENS_MEAN2, ENS_STD2, ENS_KEPT, ENS_UMEAN, ENS_USTD };
// Unwrapped precession phase atan2(Sz, Sy) + 2 pi turns of n particles into dst.
int launch_gather_phase(const double* Sy, const double* Sz, const int32_t* turns, int64_t n, double* dst,
                        void* stream);

// integratorType 6 (st_spectrum.cu): the noise spectrum.  Per parameter set,
// the Floquet frequencies of the Goertzel aggregators, the per-sample
// constants 2 cos(w dt) and sin(w dt) as the reference evaluates them (on the
// host), dt, and the test-noise amplitudes and frequencies; per particle, the
// aggregators of the last window, field-major: s1[(k * 3 + c) * n + i].
constexpr int kSpecFreqs = 17;
constexpr int kSpecBlock = 128;  // four particles (warps) per block
struct SpecSet {
  double freq[kSpecFreqs], two_cos[kSpecFreqs], sin_a[kSpecFreqs];
  double fdt;
  double na[3], nw[3];
};
struct SpecArgs {
  const SpecSet* sets;
  double *s1, *s2, *im;
  int64_t* nsamp;
};
// floquet_diagonalize's frequencies and dt (host); -1 when w gives no period.
int floquet_frequencies(const st_options& o, double freq[kSpecFreqs], double* dt);
int build_spec_set(const st_options& o, SpecSet* q);
int launch_spectrum(const RunArgs& a, int window, double next_t, const SpecArgs& sp, void* stream);

// Host-side launch helpers implemented in st_kernels.cu.  Return a cudaError_t
// cast to int (0 = success).
int launch_prepare_sets(SetParams* sets, int nsets, void* stream);
int launch_init(const RunArgs& a, int block, void* stream);
int launch_plain_window(const RunArgs& a, int window, int block, void* stream);
int launch_pack_snapshot(const RunArgs& a, int slot, void* stream);
int launch_persistent(const RunArgs& a, int variant, int blocks, int block, void* stream);
int launch_until(const RunArgs& a, double next_t, int block, void* stream);
int launch_arm_deadline(RunStatus* status, unsigned long long budget_ns, void* stream);
int probe_fp64(int sm_count, int iters, double* seconds, double* flops);
int persistent_variant_count();
// Host helpers shared across the library's translation units.
int build_set_params(const st_options& o, int64_t first, SetParams* P);
int set_last_error(int code, const char* msg);
// kind: bit 0 some set has type 2-5 (the EXT kernels), bit 1 some set has RK45
int persistent_max_blocks_per_sm(int variant, int kind);
int persistent_prepare(int variant);
int persistent_variant_block(int variant);
// 0 flattened, 1 trajectory-ahead, 2 warp-specialised, 3 three lanes per particle
int persistent_variant_family(int variant);
const char* persistent_variant_name(int variant);

}  // namespace st
