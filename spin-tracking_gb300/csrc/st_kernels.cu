// Kernels of the hot path and their launch helpers.  The window kernels
// (k_plain, k_persistent, k_batched) are templates in st_engine.cuh; this
// file instantiates them for integrator types 0 and 1, st_kernels_ext.cu with
// types 2-5.
//
//  k_init        initParticles: seed + position + velocity + gas clock, one
//                thread per particle (src/particle.cpp:638-710).
//  k_plain       runSimulation(nextTOut): one thread per particle advances its
//                particle to the window end with the reference's nested loops
//                (segment loop, step loop), one launch per output window
//                (src/particle.cpp:525-635, 865-876).
//  k_persistent  the flattened engine: a persistent grid whose lanes pull
//                particles (of any parameter set) from a device work queue and
//                run them through all requested windows; every iteration of a
//                lane's loop is one step attempt (a lane whose segment ended
//                does its trajectory event inline and rejoins).
//  k_batched     the trajectory-ahead engine (the default): as k_persistent,
//                but each lane keeps a shared-memory ring of upcoming segments,
//                produced warp-synchronously ahead of the spin, so the step loop
//                rarely leaves the converged path.  Template switches: the
//                adjoint's tape, gas collisions, stage storage, types 2-5.
//  k_pack        copies the state into one snapshot block (plain path).
#include <cuda_runtime.h>
#include <stdint.h>

#include "st_engine.cuh"
#include "st_split.cuh"
#include "st_tpp.cuh"

namespace st {

__global__ void k_arm(RunStatus* st, unsigned long long budget_ns) { st->deadline_ns = globaltimer_ns() + budget_ns; }

// ------------------------------------------------------------------ set constants
__global__ void k_prepare_sets(SetParams* sets, int nsets) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nsets) prepare_set(sets[k]);
}

// ------------------------------------------------------------------ init
__global__ void k_init(RunArgs a) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.s.n) return;
  const SetParams& P = a.sets[a.s.set[i]];
  const PState p = init_particle(P, (unsigned int)(i - P.first));
  store_state(a.s, i, p);
  a.s.w_done[i] = 0;
}

// ------------------------------------------------------------------ pack
__global__ void k_pack(RunArgs a, int slot) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.s.n) return;
  char* b = a.snap + (size_t)slot * a.snap_layout.bytes;
  const size_t* o = a.snap_layout.off;
  reinterpret_cast<double*>(b + o[0])[i] = a.s.t[i];
  reinterpret_cast<double*>(b + o[1])[i] = a.s.px[i];
  reinterpret_cast<double*>(b + o[2])[i] = a.s.py[i];
  reinterpret_cast<double*>(b + o[3])[i] = a.s.pz[i];
  reinterpret_cast<double*>(b + o[4])[i] = a.s.vx[i];
  reinterpret_cast<double*>(b + o[5])[i] = a.s.vy[i];
  reinterpret_cast<double*>(b + o[6])[i] = a.s.vz[i];
  reinterpret_cast<double*>(b + o[7])[i] = a.s.Sx[i];
  reinterpret_cast<double*>(b + o[8])[i] = a.s.Sy[i];
  reinterpret_cast<double*>(b + o[9])[i] = a.s.Sz[i];
  reinterpret_cast<int32_t*>(b + o[10])[i] = a.s.fail[i];
  reinterpret_cast<uint64_t*>(b + o[11])[i] = a.s.n_coll[i];
  reinterpret_cast<uint64_t*>(b + o[12])[i] = a.s.n_bounce[i];
  reinterpret_cast<uint64_t*>(b + o[13])[i] = a.s.n_steps[i];
  reinterpret_cast<int32_t*>(b + o[14])[i] = a.s.turns[i];
}

// ------------------------------------------------------------------ libm replacements
// The trajectory's correctly rounded functions over an array (for tests):
// fn 0 log, 1 sin, 2 cos, 3 acos.
__global__ void k_crmath_eval(int fn, const double* x, double* y, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  double s, c;
  if (fn >= 8) {  // the accurate paths alone
    y[i] = crm::cr_accurate_only(fn - 8, v);
    return;
  }
  switch (fn) {
    case 0: y[i] = crm::cr_log(v); break;
    case 1: crm::cr_sincos(v, s, c); y[i] = s; break;
    case 2: crm::cr_sincos(v, s, c); y[i] = c; break;
    case 3: y[i] = crm::cr_acos(v); break;
    default: {  // the reflection's sin (4) and cos (5) of phi = acos(v), as traj_event takes them
      double phi;
      crm::cr_acos_sincos(v, phi, s, c);
      y[i] = fn == 4 ? s : c;
    }
  }
}

int launch_crmath_eval(int fn, const double* x, double* y, int64_t n, void* stream) {
  if (n <= 0) return 0;
  k_crmath_eval<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(fn, x, y, n);
  return (int)cudaGetLastError();
}

// ------------------------------------------------------------------ FP64 peak probe
// Eight independent DFMA chains per thread: the FP64 pipe's issue rate, the
// denominator of the step kernels' roofline.
__global__ void k_fp64_probe(double* out, int iters, double b, double c) {
  double a0 = threadIdx.x * 1e-3, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
         a7 = a0 + 7;
  for (int k = 0; k < iters; ++k) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  const double s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

int probe_fp64(int sm_count, int iters, double* seconds, double* flops) {
  double* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(double));
  if (e) return (int)e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sm_count * 8, threads = 256;
  k_fp64_probe<<<blocks, threads>>>(d, 64, 0.9999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  k_fp64_probe<<<blocks, threads>>>(d, iters, 0.9999999, 1e-7);
  cudaEventRecord(e1);
  e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  *seconds = ms * 1e-3;
  *flops = 2.0 * 8.0 * (double)iters * (double)blocks * (double)threads;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  return e ? (int)e : (int)cudaGetLastError();
}

// ------------------------------------------------------------------ launchers
static inline int grid_for(int64_t n, int block) { return (int)((n + block - 1) / block); }

int launch_prepare_sets(SetParams* sets, int nsets, void* stream) {
  if (nsets <= 0) return 0;
  k_prepare_sets<<<(nsets + 127) / 128, 128, 0, (cudaStream_t)stream>>>(sets, nsets);
  return (int)cudaGetLastError();
}

int launch_init(const RunArgs& a, int block, void* stream) {
  if (a.s.n == 0) return 0;
  k_init<<<grid_for(a.s.n, block), block, 0, (cudaStream_t)stream>>>(a);
  return (int)cudaGetLastError();
}

template <int B>
static int plain_launch(const RunArgs& a, int window, double next_t, void* stream) {
  k_plain<B, false><<<grid_for(a.s.n, B), B, 0, (cudaStream_t)stream>>>(a, window, next_t);
  return (int)cudaGetLastError();
}

static int plain_dispatch(const RunArgs& a, int window, double next_t, int block, void* stream) {
  if (a.s.n == 0) return 0;
  if (a.any_ext) return launch_plain_ext(a, window, next_t, block, stream);
  // numPerGPUBlock of the reference picks the block; round to a compiled size
  if (block <= 32) return plain_launch<32>(a, window, next_t, stream);
  if (block <= 64) return plain_launch<64>(a, window, next_t, stream);
  if (block <= 128) return plain_launch<128>(a, window, next_t, stream);
  return plain_launch<256>(a, window, next_t, stream);
}

int launch_plain_window(const RunArgs& a, int window, int block, void* stream) {
  return plain_dispatch(a, window, 0.0, block, stream);
}

int launch_until(const RunArgs& a, double next_t, int block, void* stream) {
  return plain_dispatch(a, -1, next_t, block, stream);
}

int launch_arm_deadline(RunStatus* status, unsigned long long budget_ns, void* stream) {
  k_arm<<<1, 1, 0, (cudaStream_t)stream>>>(status, budget_ns);
  return (int)cudaGetLastError();
}

int launch_pack_snapshot(const RunArgs& a, int slot, void* stream) {
  if (a.s.n == 0) return 0;
  k_pack<<<grid_for(a.s.n, 256), 256, 0, (cudaStream_t)stream>>>(a, slot);
  return (int)cudaGetLastError();
}

// Persistent-kernel variants.  Family 0: the flattened kernel (k_persistent);
// family 1: the trajectory-ahead kernel (k_batched) with its ring capacity
// and top-up thresholds (start when this many lanes have room, keep filling
// while this many still have room); family 2: the warp-specialised
// trajectory-ahead kernel (k_split, block = consumer warps + one producer
// warp, ring capacity per particle; integrator types 0 and 1 only); family 3:
// three lanes per particle (k_tpp3, the flattened loop shape; types 0 and 1,
// the linear grad hook and the z cosine pulse).  Block threads and the minimum
// resident blocks per SM set the register budget.
struct Variant {
  int family, block, minb, qcap, tstart, tkeep, defer, stages;
  const char* name;
  int cw, pw, creg, preg;  // family 2: consumer and producer warps, their register shares (0: no split)
};
static const Variant kVariants[] = {
    {0, 128, 1, 0, 0, 0, 0, 0, "flat_b128_m1"},  {0, 128, 2, 0, 0, 0, 0, 0, "flat_b128_m2"},
    {0, 128, 3, 0, 0, 0, 0, 0, "flat_b128_m3"},  {0, 64, 4, 0, 0, 0, 0, 0, "flat_b64_m4"},
    {0, 256, 1, 0, 0, 0, 0, 0, "flat_b256_m1"},  {1, 128, 1, 6, 24, 16, 12, 0, "ahead_b128_q6_t24_d12"},
    {1, 128, 1, 6, 16, 12, 12, 0, "ahead_b128_q6_t16_d12"}, {1, 128, 2, 4, 24, 16, 12, 0, "ahead_b128_q4_t24_d12"},
    {1, 64, 2, 8, 24, 16, 12, 0, "ahead_b64_q8_t24_d12"},   {1, 64, 2, 8, 24, 16, 6, 0, "ahead_b64_q8_t24_d6"},
    {1, 64, 2, 8, 24, 16, 18, 0, "ahead_b64_q8_t24_d18"},   {1, 64, 2, 8, 28, 20, 12, 0, "ahead_b64_q8_t28_d12"},
    {1, 64, 2, 8, 28, 20, 12, 1, "ahead_b64_q8_t28_d12_ksmem"},
    {1, 64, 5, 6, 28, 20, 12, 1, "ahead_b64_m5_q6_t28_d12_ksmem"},
    {2, 128, 2, 8, 0, 0, 0, 0, "split_c3p1_q8", 3, 1, 0, 0},
    {2, 256, 1, 8, 0, 0, 0, 0, "split_c6p2_q8", 6, 2, 0, 0},
    {2, 384, 1, 8, 0, 0, 0, 0, "split_c8p4_q8_r184_136", 8, 4, 184, 136},
    {3, 128, 2, 0, 0, 0, 0, 0, "tpp3_b128_m2"},    {3, 128, 3, 0, 0, 0, 0, 0, "tpp3_b128_m3"},
    {1, 128, 1, 6, 16, 12, 16, 0, "ahead_b128_q6_t16_d16"}, {1, 64, 2, 8, 24, 16, 16, 0, "ahead_b64_q8_t24_d16"},
    {1, 64, 2, 12, 24, 16, 12, 0, "ahead_b64_q12_t24_d12"}, {1, 64, 2, 12, 28, 20, 16, 0, "ahead_b64_q12_t28_d16"},
    {1, 64, 2, 12, 20, 12, 12, 0, "ahead_b64_q12_t20_d12"}, {1, 64, 2, 12, 16, 8, 12, 0, "ahead_b64_q12_t16_d12"},
};
constexpr int kNumVariants = sizeof(kVariants) / sizeof(kVariants[0]);

int persistent_variant_count() { return kNumVariants; }
int persistent_variant_block(int v) { return (v >= 0 && v < kNumVariants) ? kVariants[v].block : 0; }
int persistent_variant_family(int v) { return (v >= 0 && v < kNumVariants) ? kVariants[v].family : -1; }
const char* persistent_variant_name(int v) { return (v >= 0 && v < kNumVariants) ? kVariants[v].name : "?"; }

template <bool GAS>
static const void* variant_fn_g(int v) {
  switch (v) {
    case 0: return reinterpret_cast<const void*>(&k_persistent<128, 1, false>);
    case 1: return reinterpret_cast<const void*>(&k_persistent<128, 2, false>);
    case 2: return reinterpret_cast<const void*>(&k_persistent<128, 3, false>);
    case 3: return reinterpret_cast<const void*>(&k_persistent<64, 4, false>);
    case 4: return reinterpret_cast<const void*>(&k_persistent<256, 1, false>);
    case 5:
    case 6:
    case 19: return reinterpret_cast<const void*>(&k_batched<128, 1, 6, false, GAS, 0, false>);
    case 7: return reinterpret_cast<const void*>(&k_batched<128, 2, 4, false, GAS, 0, false>);
    case 12: return reinterpret_cast<const void*>(&k_batched<64, 2, 8, false, GAS, 1, false>);
    case 13: return reinterpret_cast<const void*>(&k_batched<64, 5, 6, false, GAS, 1, false>);
    case 14: return reinterpret_cast<const void*>(&k_split<3, 1, 2, 8, GAS, 0, 0>);
    case 15: return reinterpret_cast<const void*>(&k_split<6, 2, 1, 8, GAS, 0, 0>);
#if ST_TRAJ_CORRECTLY_ROUNDED
    case 16: return reinterpret_cast<const void*>(&k_split<8, 4, 1, 8, GAS, 184, 136>);
#else
    case 16: return nullptr;  // ptxas 13.0 crashes on this instantiation with CUDA's inline log/sin/cos/acos
#endif
#if ST_GRAD_IS_LINEAR && ST_PULSE_IS_Z_COS
    case 17: return reinterpret_cast<const void*>(&k_tpp3<128, 2>);
    case 18: return reinterpret_cast<const void*>(&k_tpp3<128, 3>);
#else
    case 17:
    case 18: return nullptr;  // the three-lane step assumes the default field hooks
#endif
    case 21:
    case 22:
    case 23:
    case 24: return reinterpret_cast<const void*>(&k_batched<64, 2, 12, false, GAS, 0, false>);
    default: return reinterpret_cast<const void*>(&k_batched<64, 2, 8, false, GAS, 0, false>);  // 8 to 11, 20
  }
}
// The kernel of variant v: with gas collisions or without, and with
// integrator types 2-5 (whose instantiations handle gas and every type).
// kind: bit 0 some set has type 2-5, bit 1 some set has RK45.
static const void* variant_fn(int v, bool gas, int kind) {
  if (kind & 1) return kVariants[v].family >= 2 ? nullptr : variant_fn_ext(v);  // no k_split, k_tpp3 for types 2-5
  if ((kind & 2) && kVariants[v].family == 3) return nullptr;                  // k_tpp3 integrates DOP853 only
  return gas ? variant_fn_g<true>(v) : variant_fn_g<false>(v);
}

// Rings (records and flags), then the stage derivatives when they live in
// shared memory (10 stages x 3 components x block).
static size_t batched_smem(int block, int qcap, int stages) {
  const size_t ring = (size_t)qcap * block * kRecF * sizeof(double) + (size_t)(qcap * block + 1) / 2 * sizeof(double);
  return ring + (stages ? (size_t)30 * block * sizeof(double) : 0);
}

static int split_consumer_warps(int v) { return kVariants[v].cw; }

// A register split must fit the registers the block is launched with, and
// setmaxnreg may only raise the consumers' and lower the producers' count:
// checked against the compiled kernel before it can ever run (a split that
// does not fit would wait for registers forever).
static bool split_fits(int v, const void* fn) {
  const Variant& x = kVariants[v];
  if (x.family != 2 || x.creg == 0) return true;
  cudaFuncAttributes at{};
  if (cudaFuncGetAttributes(&at, fn) != cudaSuccess) return false;
  const long long launched = (long long)x.block * at.numRegs;
  const long long shares = 32LL * ((long long)x.cw * x.creg + (long long)x.pw * x.preg);
  return at.numRegs >= x.preg && at.numRegs <= x.creg && shares <= launched;
}

static size_t variant_smem(int v) {
  const Variant& x = kVariants[v];
  if (x.family == 0 || x.family == 3) return 0;
  if (x.family == 2) return split_smem_bytes(split_consumer_warps(v), x.qcap);
  return batched_smem(x.block, x.qcap, x.stages);
}

// Function attributes are set per device: remember which devices have them
// (devices beyond the table are set every time).
constexpr int kAttrDevices = 16;
static int current_device() {
  int d = 0;
  return cudaGetDevice(&d) == cudaSuccess ? d : kAttrDevices;
}

// Opt the kernels that need more than 48 KiB of dynamic shared memory in, once per device.
static cudaError_t ensure_smem(int v, bool gas, int kind) {
  const bool ext = (kind & 1) != 0;
  static bool done[kAttrDevices][kNumVariants][3] = {};
  const int k = ext ? 2 : (gas ? 1 : 0), d = current_device();
  if (d < kAttrDevices && done[d][v][k]) return cudaSuccess;
  const size_t sm = variant_smem(v);
  const void* fn = variant_fn(v, gas, kind);
  cudaError_t e = cudaSuccess;
  if (sm > 0 && fn) e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e == cudaSuccess && d < kAttrDevices) done[d][v][k] = true;
  return e;
}

// Function attributes of a variant's kernels, set before any graph capture.
int persistent_prepare(int v) {
  if (v < 0 || v >= kNumVariants) return (int)cudaErrorInvalidValue;
  cudaError_t e = ensure_smem(v, true, 0);
  if (e == cudaSuccess) e = ensure_smem(v, false, 0);
  if (e == cudaSuccess) e = ensure_smem(v, true, 1);
  return (int)e;
}

int persistent_max_blocks_per_sm(int v, int kind) {
  int nb = 0;
  if (v < 0 || v >= kNumVariants) return 0;
  // the gas and gas-free instantiations have the same launch bounds; take the one with gas
  const void* fn = variant_fn(v, true, kind);
  if (!fn || !split_fits(v, fn)) return 0;  // not instantiated for this kind of run, or its split does not fit
  if (ensure_smem(v, true, kind) != cudaSuccess) return 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kVariants[v].block, variant_smem(v));
  return nb;
}

int launch_persistent(const RunArgs& a, int v, int blocks, int block, void* stream) {
  if (a.s.n == 0) return 0;
  if (v < 0 || v >= kNumVariants) return (int)cudaErrorInvalidValue;
  (void)block;
  const Variant& x = kVariants[v];
  const bool gas = a.any_gas != 0;
  const int kind = (a.any_ext ? 1 : 0) | (a.any_rk45 ? 2 : 0);
  cudaError_t e = ensure_smem(v, gas, kind);
  if (e != cudaSuccess) return (int)e;
  RunArgs args = a;
  int t0 = x.tstart, t1 = x.tkeep, dk = x.defer;
  TapeArgs none{};
  void* params_flat[] = {&args};
  void* params_ahead[] = {&args, &t0, &t1, &dk, &none};
  const void* fn = variant_fn(v, gas, kind);
  if (!fn) return (int)cudaErrorInvalidValue;
  if (!split_fits(v, fn)) return (int)cudaErrorInvalidConfiguration;
  e = cudaLaunchKernel(fn, dim3(blocks), dim3(x.block), x.family == 1 ? params_ahead : params_flat, variant_smem(v),
                       (cudaStream_t)stream);
  return (int)e;
}

// The record pass of the adjoint: the trajectory-ahead kernel with its tape on
// (one configuration: kTapeBlock lanes, kTapeQcap-record rings, top-up at 24 /
// 16 lanes); the EXT instantiation (st_kernels_ext.cu) records Magnus steps.
static const void* tape_fn(bool gas, bool ext) {
  if (ext) return tape_fn_ext();
  return gas ? reinterpret_cast<const void*>(&k_batched<kTapeBlock, 1, kTapeQcap, true, true, 0, false>)
             : reinterpret_cast<const void*>(&k_batched<kTapeBlock, 1, kTapeQcap, true, false, 0, false>);
}
static size_t tape_smem() { return batched_smem(kTapeBlock, kTapeQcap, 0); }

static cudaError_t tape_ensure_smem(bool gas, bool ext) {
  static bool done[kAttrDevices][3] = {};
  const int k = ext ? 2 : (gas ? 1 : 0), d = current_device();
  if (d < kAttrDevices && done[d][k]) return cudaSuccess;
  cudaError_t e =
      cudaFuncSetAttribute(tape_fn(gas, ext), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tape_smem());
  if (e == cudaSuccess && d < kAttrDevices) done[d][k] = true;
  return e;
}

int tape_record_block() { return kTapeBlock; }

int tape_record_max_blocks_per_sm(int ext) {
  int nb = 0;
  if (tape_ensure_smem(true, ext != 0) != cudaSuccess) return 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, tape_fn(true, ext != 0), kTapeBlock, tape_smem());
  return nb;
}

int launch_tape_record(const RunArgs& a, const TapeArgs& t, int blocks, void* stream) {
  if (a.nitems == 0) return 0;
  const bool gas = a.any_gas != 0, ext = a.any_ext != 0;
  cudaError_t e = tape_ensure_smem(gas, ext);
  if (e != cudaSuccess) return (int)e;
  RunArgs args = a;
  TapeArgs tape = t;
  int t0 = 24, t1 = 16, dk = 12;
  void* params[] = {&args, &t0, &t1, &dk, &tape};
  return (int)cudaLaunchKernel(tape_fn(gas, ext), dim3(blocks), dim3(kTapeBlock), params, tape_smem(),
                               (cudaStream_t)stream);
}

}  // namespace st