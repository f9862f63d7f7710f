// Allocation-free run of the batched persistent kernel (st_run_noalloc).
//
// Some callers cannot allocate device memory themselves at the point where
// they run the tracker: a host application whose memory pool owns the whole
// GPU (a framework caching allocator, a plugin host that hands out buffers),
// or a driver that must not call cudaMalloc/cudaFree on its hot path because
// those calls synchronise the device.  st_run_noalloc lets such a caller pass
// one pre-allocated device buffer for the particle state (input and output)
// and nothing else: the small scratch the persistent kernel needs (its work
// queue cursor, work counters and the device copy of the parameter table)
// lives in the file-scope array below, which every GPU that loads the library
// holds until the process exits.
//
// Limits and rules:
//  * at most kNoAllocMaxSets parameter sets per call (the scratch is
//    kNoAllocScratchBytes = 8 KiB); more are rejected with ST_ERR_ARG;
//  * all calls on a device share the one scratch array and it keeps the last
//    call's contents; every call clears the parts that must start at zero
//    before launching, so calls that overlap on the GPU (different streams or
//    host threads at once) race on it and must not be issued;
//  * the first call on each device (and again after that device's primary
//    context was reset) looks up the array's device address with
//    cudaGetSymbolAddress, with that device current; make that first call
//    before any stream capture;
//  * the launch is fixed: the flattened persistent kernel (flat_b128_m2)
//    with as many 128-thread blocks per SM as its occupancy allows, without
//    the autotuner or the type-grouped work order of st_run_windows (both
//    allocate); results are the same, throughput can be lower.
#include <cuda_runtime.h>

#include <mutex>
#include <stdint.h>
#include <string>

#include "spintrack.h"
#include "st_internal.h"

namespace st {

constexpr int kNoAllocMaxSets = 8;
constexpr int kNoAllocVariant = 1;  // flat_b128_m2: flattened persistent kernel, 128 threads, >= 2 blocks per SM
constexpr size_t kNoAllocScratchBytes = 8192;
constexpr size_t kNoAllocStatusBytes = 256;  // RunStatus, padded
static_assert(sizeof(RunStatus) <= kNoAllocStatusBytes, "status block");
static_assert(kNoAllocStatusBytes + kNoAllocMaxSets * sizeof(SetParams) <= kNoAllocScratchBytes, "scratch size");

// The scratch: [0, 256) run status, [256, ...) parameter table.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};
void* g_scratch_ctx[kMaxDevices] = {};  // the context the address was looked up in

// The current driver context (CUcontext), fetched through the runtime's driver
// entry point so the library does not link libcuda directly.  A primary
// context that was reset (cudaDeviceReset) comes back as a new context, in
// which the module is loaded again and the array may sit at another address.
typedef int (*CtxGetCurrentFn)(void**);
void* current_context() {
  static CtxGetCurrentFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrentFn>(f);
  }();
  void* ctx = nullptr;
  if (!fn || fn(&ctx) != 0) return nullptr;
  return ctx;
}

// Device address of the scratch array on the current device.  In host code the
// array's name is only a stand-in for the symbol, never a usable pointer.  The
// address is looked up once per device and context; before the runtime's first
// call on a device no context is current yet, and the lookup itself makes the
// primary context current.
int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return set_last_error(ST_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  void* ctx = current_context();
  if (!g_scratch_addr[device] || !ctx || ctx != g_scratch_ctx[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      return set_last_error(ST_ERR_CUDA, (std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e)).c_str());
    }
    g_scratch_addr[device] = p;
    // the runtime has made the primary context current by now
    g_scratch_ctx[device] = ctx ? ctx : current_context();
  }
  *out = static_cast<unsigned char*>(g_scratch_addr[device]);
  return ST_OK;
}

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Caller buffer layout: the state arrays in this order, each n elements,
// each starting on a 256-byte boundary.
constexpr int kNumFields = 28;
constexpr size_t kElem[kNumFields] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8,  // t pos_xyz v_xyz S_xyz
                                      4, 8, 8, 8,                    // fail n_coll n_bounce n_steps
                                      8, 8,                          // h next_gas
                                      8, 8, 8, 8, 8, 1,              // rng x y z w spare has
                                      1, 1, 1,                       // stop coll wall
                                      4, 4, 4};                      // set w_done turns

size_t state_bytes(int64_t n) {
  const size_t m = (size_t)(n > 0 ? n : 1);
  size_t b = 0;
  for (int k = 0; k < kNumFields; ++k) b += align256(kElem[k] * m);
  return b;
}

DeviceState carve(void* base, int64_t n) {
  const size_t m = (size_t)(n > 0 ? n : 1);
  char* p = static_cast<char*>(base);
  void* f[kNumFields];
  for (int k = 0; k < kNumFields; ++k) {
    f[k] = p;
    p += align256(kElem[k] * m);
  }
  DeviceState s;
  s.n = n;
  s.t = (double*)f[0];
  s.px = (double*)f[1]; s.py = (double*)f[2]; s.pz = (double*)f[3];
  s.vx = (double*)f[4]; s.vy = (double*)f[5]; s.vz = (double*)f[6];
  s.Sx = (double*)f[7]; s.Sy = (double*)f[8]; s.Sz = (double*)f[9];
  s.fail = (int32_t*)f[10];
  s.n_coll = (uint64_t*)f[11]; s.n_bounce = (uint64_t*)f[12]; s.n_steps = (uint64_t*)f[13];
  s.h = (double*)f[14]; s.next_gas = (double*)f[15];
  s.rx = (uint64_t*)f[16]; s.ry = (uint64_t*)f[17]; s.rz = (uint64_t*)f[18]; s.rw = (uint64_t*)f[19];
  s.rspare = (double*)f[20]; s.rhas = (uint8_t*)f[21];
  s.stop = (uint8_t*)f[22]; s.coll = (uint8_t*)f[23]; s.wall = (uint8_t*)f[24];
  s.set = (int32_t*)f[25]; s.w_done = (int32_t*)f[26]; s.turns = (int32_t*)f[27];
  return s;
}

// Set index of every particle from the parameter table in the scratch.
__global__ void k_noalloc_sets(DeviceState s, const SetParams* sets, int nsets) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= s.n) return;
  int k = 0;
  while (k + 1 < nsets && i >= sets[k + 1].first) ++k;
  s.set[i] = k;
}

}  // namespace
}  // namespace st

extern "C" int st_run_noalloc(const st_options* sets, int nsets, void* state, size_t* state_bytes_io, int w_end,
                              void* stream) {
  using namespace st;
  if (!sets || !state_bytes_io) return set_last_error(ST_ERR_ARG, "st_run_noalloc: null argument");
  if (nsets < 1 || nsets > kNoAllocMaxSets)
    return set_last_error(ST_ERR_ARG, "st_run_noalloc: 1 to 8 parameter sets per call (8 KiB device scratch)");
  SetParams table[kNoAllocMaxSets];
  int64_t n = 0;
  for (int k = 0; k < nsets; ++k) {
    if (sets[k].integratorType == 6)
      return set_last_error(ST_ERR_UNSUPPORTED, "st_run_noalloc: integratorType 6 keeps per-particle spectra; use st_create");
    const int r = build_set_params(sets[k], n, &table[k]);
    if (r != ST_OK) return r;
    n += sets[k].numParticles;
  }
  const size_t need = state_bytes(n);
  if (!state) {  // size query
    *state_bytes_io = need;
    return ST_OK;
  }
  if (*state_bytes_io < need) return set_last_error(ST_ERR_ARG, "st_run_noalloc: state buffer smaller than required");
  if (((uintptr_t)state & 255u) != 0) return set_last_error(ST_ERR_ARG, "st_run_noalloc: state must be 256-byte aligned");
  if (w_end < 0) return set_last_error(ST_ERR_ARG, "st_run_noalloc: negative window count");
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return set_last_error(ST_ERR_CUDA, cudaGetErrorString(e));
  unsigned char* scratch = nullptr;
  int r = scratch_address(device, &scratch);
  if (r != ST_OK) return r;
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return set_last_error(ST_ERR_CUDA, cudaGetErrorString(e));
  cudaStream_t st_ = static_cast<cudaStream_t>(stream);
  RunStatus* status = reinterpret_cast<RunStatus*>(scratch);
  SetParams* params = reinterpret_cast<SetParams*>(scratch + kNoAllocStatusBytes);
  // clear the run status (queue cursor, counters, deadline) and upload the table
  e = cudaMemsetAsync(status, 0, sizeof(RunStatus), st_);
  if (e == cudaSuccess) e = cudaMemcpyAsync(params, table, sizeof(SetParams) * nsets, cudaMemcpyHostToDevice, st_);
  if (e != cudaSuccess) return set_last_error(ST_ERR_CUDA, cudaGetErrorString(e));
  RunArgs a{};
  a.sets = params;
  a.nsets = nsets;
  a.order = nullptr;
  a.nitems = n;
  a.s = carve(state, n);
  a.status = status;
  a.snap = nullptr;
  a.w_begin = 0;
  a.w_end = w_end;
  a.deadline_armed = 0;
  a.count_work = 1;
  a.any_gas = 1;  // the caller's sets are not inspected on the host: the kernel with gas handles any set
  a.any_ext = 0;
  a.any_rk45 = 0;
  for (int k = 0; k < nsets; ++k) {
    a.any_ext |= (sets[k].integratorType >= 2 && sets[k].integratorType <= 5) ? 1 : 0;
    a.any_rk45 |= sets[k].integratorType == 1 ? 1 : 0;
  }
  if (int pe = launch_prepare_sets(params, nsets, st_)) return set_last_error(ST_ERR_CUDA, cudaGetErrorString((cudaError_t)pe));
  if (n > 0) {
    k_noalloc_sets<<<(unsigned)((n + 255) / 256), 256, 0, st_>>>(a.s, params, nsets);
    e = cudaGetLastError();
    if (e != cudaSuccess) return set_last_error(ST_ERR_CUDA, cudaGetErrorString(e));
    // flat_b128_m2 (the flattened persistent kernel) at its full occupancy; the
    // occupancy query and the shared-memory attribute allocate nothing
    const int per_sm = persistent_max_blocks_per_sm(kNoAllocVariant, a.any_ext | (a.any_rk45 << 1));
    if (per_sm < 1) return set_last_error(ST_ERR_CUDA, "st_run_noalloc: the persistent kernel cannot be resident");
    int le = launch_init(a, 256, st_);
    if (!le) le = launch_persistent(a, kNoAllocVariant, sms * per_sm, 0, st_);
    if (le) return set_last_error(ST_ERR_CUDA, cudaGetErrorString((cudaError_t)le));
  }
  RunStatus h{};
  e = cudaMemcpyAsync(&h, status, sizeof(RunStatus), cudaMemcpyDeviceToHost, st_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
  if (e != cudaSuccess) return set_last_error(ST_ERR_CUDA, (std::string("kernel execution: ") + cudaGetErrorString(e)).c_str());
  *state_bytes_io = need;
  // the same status checks as the allocating path's run end
  if (h.pad) return set_last_error(ST_ERR_CUDA, "internal: a persistent-kernel lane could not make progress");
  if (h.deadline_hit) return set_last_error(ST_ERR_DEADLINE, "device time budget ran out");
  return ST_OK;
}
