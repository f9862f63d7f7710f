// Host library behind include/spintrack.h: options parsing, the engine
// context (device state, parameter-set table, stream), the window driver and
// the format-'A' writer.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "spintrack.h"
#include "st_fields.cuh"
#include "st_internal.h"

using st::SetParams;

static_assert(sizeof(st_options) == 440, "st_options must match the reference options image");
static_assert(sizeof(st_vec3) == 24, "st_vec3 layout");

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define ST_CUDA(expr)                                                                            \
  do {                                                                                           \
    cudaError_t e_ = (expr);                                                                     \
    if (e_ != cudaSuccess) return fail(ST_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define ST_TRY(expr)            \
  do {                          \
    int r_ = (expr);            \
    if (r_ != ST_OK) return r_; \
  } while (0)

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- parsing
std::vector<std::string> split_fields(const char* line) {
  // grabElementsInLine + removeWhitespace (src/optionsParser.cpp:11-37)
  std::vector<std::string> out(1);
  for (const char* c = line; *c; ++c) {
    if (*c == ',')
      out.emplace_back();
    else if (!std::isspace(static_cast<unsigned char>(*c)))
      out.back().push_back(*c);
  }
  return out;
}

bool to_double(const std::string& s, double* v) {
  if (s.empty()) return false;
  char* end = nullptr;
  errno = 0;
  const double x = std::strtod(s.c_str(), &end);
  if (end == s.c_str()) return false;  // no conversion: leave the option unchanged
  *v = x;
  return true;
}

bool to_int(const std::string& s, int* v) {
  if (s.empty()) return false;
  char* end = nullptr;
  errno = 0;
  long x = std::strtol(s.c_str(), &end, 10);
  if (end == s.c_str() || errno == ERANGE || x > 2147483647L || x < -2147483648L) return false;
  *v = (int)x;
  return true;
}

// to_bool (src/optionsParser.cpp:16-22): boolalpha extraction of the lowered
// token, so a leading "true" gives true and anything else false.
bool to_bool(const std::string& s) {
  std::string low;
  for (char c : s) low.push_back((char)std::tolower(static_cast<unsigned char>(c)));
  return low.compare(0, 4, "true") == 0;
}

// ---------------------------------------------------------------- params
int build_params(const st_options& o, int64_t first, SetParams* P) {
  if (o.numParticles < 0) return fail(ST_ERR_ARG, "numParticles must be >= 0");
  if (o.integratorType == 6 && !(o.w != 0.0 && std::isfinite(o.w)))
    return fail(ST_ERR_ARG, "integratorType 6 needs a nonzero pulse frequency w: its Floquet period is 2 pi / w");
  if (o.dist != 'C' && o.dist != 'M')
    return fail(ST_ERR_UNSUPPORTED, std::string("dist must be 'C' or 'M', got '") + o.dist + "'");
  if (!(o.ioutInt > 0.0)) return fail(ST_ERR_ARG, "ioutInt must be > 0");
  std::memset(P, 0, sizeof(*P));
  P->Lx = o.L.x; P->Ly = o.L.y; P->Lz = o.L.z;
  P->maxPosStep = o.maxPosStep;
  P->tc = o.tc;
  P->sqrtKT_m = o.sqrtKT_m;
  P->diffuse = o.diffuse;
  P->V = o.V;
  P->gamma = o.gamma;
  P->B0x = o.B0.x; P->B0y = o.B0.y; P->B0z = o.B0.z;
  P->Ex = o.E.x; P->Ey = o.E.y; P->Ez = o.E.z;
  P->Gx[0] = o.Gx.x; P->Gx[1] = o.Gx.y; P->Gx[2] = o.Gx.z;
  P->Gy[0] = o.Gy.x; P->Gy[1] = o.Gy.y; P->Gy[2] = o.Gy.z;
  P->Gz[0] = o.Gz.x; P->Gz[1] = o.Gz.y; P->Gz[2] = o.Gz.z;
  P->a = o.a;
  P->w = o.w;
  P->inv_c2 = 1.0 / st::kC2;
  P->rtol = o.rtol; P->atol = o.atol; P->hmin = o.hmin; P->hmax = o.hmax; P->h0 = o.h;
  P->safe = o.safe; P->fac1 = o.fac1; P->fac2 = o.fac2; P->beta = o.beta;
  P->facc1 = 1.0 / o.fac1;
  P->facc2 = 1.0 / o.fac2;
  P->expo1 = 1.0 / 8.0 - o.beta * 0.2;
  P->inv_safe = 1.0 / o.safe;
  P->t0 = o.t0; P->tf = o.tf; P->ioutInt = o.ioutInt;
  P->yi_x = o.yi.x; P->yi_y = o.yi.y; P->yi_z = o.yi.z;
  P->nmax = o.nmax;
  P->seed = o.seed;
  P->integrator = o.integratorType;
  P->nwin = st_num_windows(&o);
  P->gravity = o.gravity ? 1 : 0;
  P->gas = o.gas_coll ? 1 : 0;
  P->fixed = o.fixedStepSize ? 1 : 0;
  P->keep = o.keepStepSize ? 1 : 0;
  P->dist = o.dist;
  P->first = first;
  P->n = o.numParticles;
  return ST_OK;
}

}  // namespace

// Entry points for other translation units of the library (st_noalloc.cu).
namespace st {
int build_set_params(const st_options& o, int64_t first, SetParams* P) { return build_params(o, first, P); }
int set_last_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace st

// ==================================================================== context
struct st_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<st_options> opts;
  std::vector<SetParams> sets_h;
  SetParams* sets_d = nullptr;
  int64_t n = 0;
  st::DeviceState s{};
  void* arena = nullptr;
  st::RunStatus* status_d = nullptr;
  st::RunStatus* status_h = nullptr;  // pinned
  int64_t* order_d = nullptr;
  bool initialized = false;
  bool window_grid = true;  // particles sit on window boundaries (false after st_run_until off-grid)
  st_launch_config lc{0, 0, -1};
  bool lc_tuned = false;  // lc came from the autotuner (for the sets it was tuned on)
  int sm_count = 0;
  double deadline_s = 0.0;
  st_counters last{};
  st::SnapLayout snap{};
  bool fresh = false;        // st_init ran and no run call since
  size_t arena_bytes = 0;    // bytes of one particle-state arena (state_layout)
  // CUDA graphs of st_run_windows calls, most recent last
  struct RunGraph {
    int kernel, w_begin, w_end, block, variant, bps;
    void* snap;
    double deadline_s;
    cudaGraphExec_t exec;
    int launches;
  };
  std::vector<RunGraph> graphs;
  void* ens_buf = nullptr;   // ensemble statistics: control slots, block partials, histogram
  // integratorType 6 (every set of the context): the noise-spectrum aggregators
  bool spectrum = false;
  st::SpecSet* spec_sets_d = nullptr;
  void* spec_pp = nullptr;        // s1, s2, im (17 x 3 per particle each), samples per particle
  st::SpecArgs spec{};
  // adjoint (allocated by st_adjoint_record)
  double* tape_pool = nullptr;
  int32_t* tape_prev = nullptr;
  int64_t tape_pages = 0;
  void* tape_pp = nullptr;   // per-particle tape arrays and work orders
  unsigned long long* tape_head = nullptr;
  long long* tape_error = nullptr;
  st::TapeArgs tape{};       // pointers into the above: the chains of replays (and of a record whose tape fits)
  st::TapeArgs tail{};       // the chains of the record pass's last intervals (kept when the whole tape does not fit)
  unsigned long long* tail_head = nullptr;
  int adj_tail_from = 0;          // checkpoint interval where the kept tail starts (ckpt_count: no tail)
  int64_t adj_tail_pages = 0;     // pool pages the record pass's tape holds (replays use the pages after them)
  int64_t* adj_order = nullptr;   // every particle, longest tape first
  int64_t* adj_gorder = nullptr;  // a group of particles replayed together
  void* ckpt_arena = nullptr;     // state checkpoints, ckpt_count arenas
  int ckpt_alloc = 0;
  int ckpt_every = 0, ckpt_count = 0;
  void* replay_arena = nullptr;   // state of a replay
  std::vector<int64_t> adj_nsteps_h, adj_nsegs_h;
  std::vector<uint8_t> adj_stop_h;
  double* adj_lam_buf = nullptr;  // per loss and particle: the spin adjoint carried between chunks
  size_t adj_lam_cap = 0;          // doubles allocated
  int adj_nloss = 1;               // losses of the running backward
  double* adj_grad_base = nullptr; // their gradients, loss after loss
  int adj_w_end = 0;
  int adj_w_run = 0;              // windows the record pass ran (w_end capped at the sets' windows)
  bool adj_recorded = false;
  bool adj_resident = false;      // the record pass's tape is complete and still in the pool
  st_adjoint_stats adj_stats{};
};

namespace {

// Field layout of one particle-state arena: every SoA array 256-byte
// aligned, in a fixed order.  base == nullptr only computes the size.
size_t state_layout(st::DeviceState& s, char* base, int64_t n) {
  const size_t m = (size_t)std::max<int64_t>(n, 1);
  struct Field {
    void** ptr;
    size_t elem;
  };
  Field f[] = {{(void**)&s.t, 8},        {(void**)&s.px, 8},   {(void**)&s.py, 8},     {(void**)&s.pz, 8},
               {(void**)&s.vx, 8},       {(void**)&s.vy, 8},   {(void**)&s.vz, 8},     {(void**)&s.Sx, 8},
               {(void**)&s.Sy, 8},       {(void**)&s.Sz, 8},   {(void**)&s.h, 8},      {(void**)&s.next_gas, 8},
               {(void**)&s.rx, 8},       {(void**)&s.ry, 8},   {(void**)&s.rz, 8},     {(void**)&s.rw, 8},
               {(void**)&s.rspare, 8},   {(void**)&s.rhas, 1}, {(void**)&s.fail, 4},   {(void**)&s.n_coll, 8},
               {(void**)&s.n_bounce, 8}, {(void**)&s.n_steps, 8}, {(void**)&s.stop, 1}, {(void**)&s.coll, 1},
               {(void**)&s.wall, 1},     {(void**)&s.set, 4},  {(void**)&s.w_done, 4},  {(void**)&s.turns, 4}};
  size_t off = 0;
  for (auto& x : f) {
    *x.ptr = base ? base + off : nullptr;
    off += align256(x.elem * m);
  }
  s.n = n;
  return off;
}

int ctx_alloc(st_ctx* c) {
  const int64_t n = c->n;
  const size_t m = (size_t)std::max<int64_t>(n, 1);
  st::DeviceState& s = c->s;
  const size_t total = state_layout(s, nullptr, n);
  cudaError_t e = cudaMalloc(&c->arena, total);
  if (e != cudaSuccess) return fail(ST_ERR_NOMEM, std::string("cudaMalloc state: ") + cudaGetErrorString(e));
  state_layout(s, (char*)c->arena, n);
  c->arena_bytes = total;
  s.n = n;
  ST_CUDA(cudaMemsetAsync(c->arena, 0, total, c->stream));
  // set index of every particle
  std::vector<int32_t> set_of((size_t)m, 0);
  for (size_t k = 0; k < c->sets_h.size(); ++k)
    for (int64_t j = 0; j < c->sets_h[k].n; ++j) set_of[(size_t)(c->sets_h[k].first + j)] = (int32_t)k;
  ST_CUDA(cudaMemcpyAsync(s.set, set_of.data(), 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  ST_CUDA(cudaMalloc(&c->sets_d, sizeof(SetParams) * std::max<size_t>(c->sets_h.size(), 1)));
  ST_CUDA(cudaMemcpyAsync(c->sets_d, c->sets_h.data(), sizeof(SetParams) * c->sets_h.size(), cudaMemcpyHostToDevice,
                          c->stream));
  if (int e = st::launch_prepare_sets(c->sets_d, (int)c->sets_h.size(), c->stream))
    return fail(ST_ERR_CUDA, std::string("prepare sets: ") + cudaGetErrorString((cudaError_t)e));
  ST_CUDA(cudaMalloc(&c->status_d, sizeof(st::RunStatus)));
  ST_CUDA(cudaMemsetAsync(c->status_d, 0, sizeof(st::RunStatus), c->stream));
  ST_CUDA(cudaMallocHost(&c->status_h, sizeof(st::RunStatus)));
  // snapshot block layout: kSnapFields arrays of n entries
  const size_t esz[st::kSnapFields] = {8, 8, 8, 8, 8, 8, 8, 8, 8, 8, 4, 8, 8, 8, 4};
  size_t off = 0;
  c->snap.n = n;
  for (int k = 0; k < st::kSnapFields; ++k) {
    c->snap.off[k] = off;
    off += align256(esz[k] * m);
  }
  c->snap.bytes = off;
  if (c->spectrum) {  // integratorType 6: the Floquet frequencies per set and the aggregators
    std::vector<st::SpecSet> q(c->opts.size());
    for (size_t k = 0; k < c->opts.size(); ++k)
      if (st::build_spec_set(c->opts[k], &q[k]) != 0) return fail(ST_ERR_ARG, "integratorType 6: no Floquet period");
    ST_CUDA(cudaMalloc(&c->spec_sets_d, sizeof(st::SpecSet) * q.size()));
    ST_CUDA(cudaMemcpyAsync(c->spec_sets_d, q.data(), sizeof(st::SpecSet) * q.size(), cudaMemcpyHostToDevice,
                            c->stream));
    const size_t acc = align256(sizeof(double) * 3 * st::kSpecFreqs * m);
    ST_CUDA(cudaMalloc(&c->spec_pp, 3 * acc + align256(8 * m)));
    ST_CUDA(cudaMemsetAsync(c->spec_pp, 0, 3 * acc + align256(8 * m), c->stream));
    char* b = (char*)c->spec_pp;
    c->spec.sets = c->spec_sets_d;
    c->spec.s1 = (double*)b;
    c->spec.s2 = (double*)(b + acc);
    c->spec.im = (double*)(b + 2 * acc);
    c->spec.nsamp = (int64_t*)(b + 3 * acc);
  }
  ST_CUDA(cudaStreamSynchronize(c->stream));
  return ST_OK;
}

// Work order for the persistent queue: sets grouped by integrator (the
// fourth/fifth-order ones first: RK45, RK45 and RKF45 with quaternions,
// RKF45; then Magnus, DOP853, trajectory-only), so that a warp's lanes run one
// step code and do not diverge between two; within a group, longest expected
// particles first, so the tail of the run is short.  Cost = simulated time,
// the fourth/fifth-order types weighted 2000x (at rtol 1e-12 RK45 takes ~4400x
// the attempts of DOP853, each ~0.4x the work).
// Some set integrates with type 2-5: the runs take the EXT kernels.
bool ctx_any_rk45(const st_ctx* c) {
  for (const auto& P : c->sets_h)
    if (P.integrator == 1) return true;
  return false;
}
// Which persistent-kernel instantiations a context's runs need: bit 0 some set
// has type 2-5, bit 1 some set has RK45.
int ctx_kind(const st_ctx* c);

bool ctx_any_ext(const st_ctx* c) {
  for (const auto& P : c->sets_h)
    if (P.integrator >= 2 && P.integrator <= 5) return true;
  return false;
}
int ctx_kind(const st_ctx* c) { return (ctx_any_ext(c) ? 1 : 0) | (ctx_any_rk45(c) ? 2 : 0); }

int order_group(int it) {
  switch (it) {
    case 1: return 0;
    case 3: return 1;
    case 5: return 2;
    case 4: return 3;
    case 2: return 4;
    case 0: return 5;
    default: return 6;
  }
}
double order_weight(int it) { return (it == 1 || it == 3 || it == 4 || it == 5) ? 2000.0 : 1.0; }

int ctx_build_order(st_ctx* c) {
  if (c->order_d || c->sets_h.size() <= 1) return ST_OK;
  std::vector<int> idx(c->sets_h.size());
  for (size_t k = 0; k < idx.size(); ++k) idx[k] = (int)k;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) {
    const SetParams &A = c->sets_h[a], &B = c->sets_h[b];
    const int ga = order_group(A.integrator), gb = order_group(B.integrator);
    if (ga != gb) return ga < gb;
    const double ca = order_weight(A.integrator) * A.nwin * A.ioutInt;
    const double cb = order_weight(B.integrator) * B.nwin * B.ioutInt;
    return ca > cb;
  });
  std::vector<int64_t> order;
  order.reserve((size_t)c->n);
  for (int k : idx)
    for (int64_t j = 0; j < c->sets_h[k].n; ++j) order.push_back(c->sets_h[k].first + j);
  ST_CUDA(cudaMalloc(&c->order_d, sizeof(int64_t) * std::max<size_t>(order.size(), 1)));
  ST_CUDA(cudaMemcpyAsync(c->order_d, order.data(), sizeof(int64_t) * order.size(), cudaMemcpyHostToDevice,
                          c->stream));
  return ST_OK;
}

st::RunArgs make_args(st_ctx* c, int w_begin, int w_end, void* snap) {
  st::RunArgs a{};
  a.sets = c->sets_d;
  a.nsets = (int)c->sets_h.size();
  a.order = c->order_d;
  a.nitems = c->n;
  a.s = c->s;
  a.status = c->status_d;
  a.snap = (char*)snap;
  a.snap_layout = c->snap;
  a.w_begin = w_begin;
  a.w_end = w_end;
  a.deadline_armed = 0;
  a.count_work = 1;
  a.any_gas = 0;
  a.any_ext = ctx_any_ext(c) ? 1 : 0;
  a.any_rk45 = ctx_any_rk45(c) ? 1 : 0;
  for (const auto& P : c->sets_h) a.any_gas |= P.gas ? 1 : 0;
  return a;
}

int begin_run(st_ctx* c) {
  ST_CUDA(cudaSetDevice(c->device));
  ST_CUDA(cudaMemsetAsync(c->status_d, 0, sizeof(st::RunStatus), c->stream));
  return ST_OK;
}

// Arm the device time budget: a one-thread kernel stores %globaltimer + budget.
int arm_deadline(st_ctx* c, st::RunArgs& a);

int end_run(st_ctx* c, int launches) {
  ST_CUDA(cudaMemcpyAsync(c->status_h, c->status_d, sizeof(st::RunStatus), cudaMemcpyDeviceToHost, c->stream));
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(ST_ERR_CUDA, std::string("kernel execution: ") + cudaGetErrorString(e));
  c->last.dop_attempts = c->status_h->dop_attempts;
  c->last.rk45_attempts = c->status_h->rk45_attempts;
  c->last.ext_attempts = c->status_h->ext_attempts;
  c->last.segments = c->status_h->segments;
  c->last.kernel_launches = (uint64_t)launches;
  c->last.graph_launches = 0;
  c->last.graph_captures = 0;
  if (c->status_h->pad) return fail(ST_ERR_CUDA, "internal: a persistent-kernel lane could not make progress");
  if (c->status_h->deadline_hit) return fail(ST_ERR_DEADLINE, "device time budget ran out; state saved at window ends");
  return ST_OK;
}

}  // namespace

namespace {
int arm_deadline(st_ctx* c, st::RunArgs& a) {
  if (c->deadline_s <= 0.0) return ST_OK;
  int e = st::launch_arm_deadline(c->status_d, (unsigned long long)(c->deadline_s * 1e9), c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("arm deadline: ") + cudaGetErrorString((cudaError_t)e));
  a.deadline_armed = 1;  // kernels read the armed value from the status block
  return ST_OK;
}

// Autotuner: time each persistent-kernel variant and occupancy on a sample of
// the context's own parameter sets (one window of a scratch context), keep the
// fastest.
int autotune(st_ctx* c);

int run_persistent(st_ctx* c, int w_begin, int w_end, void* snap) {
  ST_TRY(ctx_build_order(c));
  if (c->lc.variant < 0 || c->lc.blocks_per_sm <= 0) ST_TRY(autotune(c));
  st::RunArgs a = make_args(c, w_begin, w_end, snap);
  ST_TRY(arm_deadline(c, a));
  const int blocks = c->sm_count * c->lc.blocks_per_sm;
  int e = st::launch_persistent(a, c->lc.variant, blocks, c->lc.block_threads, c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("persistent launch: ") + cudaGetErrorString((cudaError_t)e));
  return ST_OK;
}

int plain_block(const st_ctx* c) {
  int b = c->opts.empty() ? 128 : c->opts[0].numPerGPUBlock;
  return b > 0 ? b : 128;
}

}  // namespace

// ==================================================================== C ABI
extern "C" {

int st_version(void) { return 1; }
const char* st_last_error(void) { return g_err.c_str(); }
size_t st_options_size(void) { return sizeof(st_options); }

void st_options_default(st_options* o) {
  std::memset(o, 0, sizeof(*o));  // padding bytes of the header image are zero
  o->B0 = {3e-6, 0.0, 0.0};
  o->E = {75e5, 0.0, 0.0};
  o->L = {0.07, 0.1, 0.4};
  o->yi = {0.0, 0.0, 1.0};
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
  o->swapStepSize = 1.0 - 4;  // the reference's default expression, -3
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

int st_parse_line(st_options* o, const char* line) {
  if (!o || !line) return fail(ST_ERR_ARG, "null argument");
  std::vector<std::string> e = split_fields(line);
  if (e.size() < 2) return fail(ST_ERR_ARG, std::string("Misunderstood input line in options file: ") + line);
  const std::string& k = e[0];
  auto num = [&](size_t i, double* v) -> bool {
    if (i >= e.size() || !to_double(e[i], v)) {
      fail(ST_ERR_ARG, "malformed number in line: " + std::string(line));
      return false;
    }
    return true;
  };
  auto vec = [&](st_vec3* v) -> int {
    double a, b, cc;
    if (!num(1, &a) || !num(2, &b) || !num(3, &cc)) return ST_ERR_ARG;
    *v = {a, b, cc};
    return ST_OK;
  };
  auto dbl = [&](double* v) -> int { return num(1, v) ? ST_OK : ST_ERR_ARG; };
  auto integer = [&](int* v) -> int {
    if (!to_int(e[1], v)) return fail(ST_ERR_ARG, "malformed integer in line: " + std::string(line));
    return ST_OK;
  };
  auto uinteger = [&](unsigned int* v) -> int {
    int x;
    if (!to_int(e[1], &x)) return fail(ST_ERR_ARG, "malformed integer in line: " + std::string(line));
    *v = (unsigned int)x;
    return ST_OK;
  };
  // keys of src/optionsParser.cpp:50-170
  if (k == "L") return vec(&o->L);
  if (k == "yi") return vec(&o->yi);
  if (k == "Gx") return vec(&o->Gx);
  if (k == "Gy") return vec(&o->Gy);
  if (k == "Gz") return vec(&o->Gz);
  if (k == "dist") {
    o->dist = e[1].empty() ? '\0' : e[1][0];
    return ST_OK;
  }
  if (k == "m") return dbl(&o->m);
  if (k == "gas_coll") { o->gas_coll = to_bool(e[1]); return ST_OK; }
  if (k == "T") return dbl(&o->T);
  if (k == "diffuse") return dbl(&o->diffuse);
  if (k == "gamma") return dbl(&o->gamma);
  if (k == "V") return dbl(&o->V);
  if (k == "a") return dbl(&o->a);
  if (k == "w") return dbl(&o->w);
  if (k == "gravity") { o->gravity = to_bool(e[1]); return ST_OK; }
  if (k == "fixedStepSize") { o->fixedStepSize = to_bool(e[1]); return ST_OK; }
  if (k == "keepStepSize") { o->keepStepSize = to_bool(e[1]); return ST_OK; }
  if (k == "B0") return vec(&o->B0);
  if (k == "E") return vec(&o->E);
  if (k == "t0") return dbl(&o->t0);
  if (k == "tf") return dbl(&o->tf);
  if (k == "rtol") return dbl(&o->rtol);
  if (k == "atol") return dbl(&o->atol);
  if (k == "beta") return dbl(&o->beta);
  if (k == "uround") return dbl(&o->uround);
  if (k == "safe") return dbl(&o->safe);
  if (k == "fac1") return dbl(&o->fac1);
  if (k == "fac2") return dbl(&o->fac2);
  if (k == "hmax") return dbl(&o->hmax);
  if (k == "hmin") return dbl(&o->hmin);
  if (k == "h") return dbl(&o->h);
  if (k == "nmax") return uinteger(&o->nmax);
  if (k == "seed") return uinteger(&o->seed);
  if (k == "maxPosStep") return dbl(&o->maxPosStep);
  if (k == "integratorType") return integer(&o->integratorType);
  if (k == "swapStepSize") return dbl(&o->swapStepSize);
  if (k == "numParticles") return integer(&o->numParticles);
  if (k == "numPerGPUBlock") return integer(&o->numPerGPUBlock);
  if (k == "ioutInt") return dbl(&o->ioutInt);
  if (k == "iout") return integer(&o->iout);
  g_err = "Unrecognized Option: " + k + " (line ignored)";
  return 1;
}

int st_parse_params(const char* path, st_options* o) {
  if (!o || !path) return fail(ST_ERR_ARG, "null argument");
  st_options_default(o);
  FILE* f = std::fopen(path, "r");
  if (!f) return fail(ST_ERR_IO, std::string("cannot open params file ") + path + " (defaults kept)");
  std::string line;
  int c;
  int lineno = 0;
  int rc = ST_OK;
  auto flush = [&]() {
    ++lineno;
    int r = st_parse_line(o, line.c_str());
    if (r == 1) {
      std::fprintf(stderr, "Unrecognized Option: %s\nLine Ignored\n", split_fields(line.c_str())[0].c_str());
    } else if (r != ST_OK) {
      const std::vector<std::string> e = split_fields(line.c_str());
      if (e.size() >= 2 && rc == ST_OK) {
        rc = fail(ST_ERR_ARG, std::string(path) + ":" + std::to_string(lineno) + ": " + g_err);
      }
      // lines with fewer than two fields are skipped, as the reference does
    }
    line.clear();
  };
  while ((c = std::fgetc(f)) != EOF) {
    if (c == '\n')
      flush();
    else
      line.push_back((char)c);
  }
  if (!line.empty()) flush();
  std::fclose(f);
  return rc;
}

void st_derive(st_options* o) {
  const double k = 1.380649e-23;  // src/simulation.cpp:9-11
  o->tc = 1.6e-4 * o->m / (k * std::pow(o->T, 8.0));
  o->sqrtKT_m = std::sqrt(k * o->T / o->m);
}

int st_num_windows(const st_options* o) {
  const double q = std::floor((double)(o->tf - o->t0) / o->ioutInt);
  if (!(q > 0.0)) return 0;
  if (q > 2147483647.0) return 2147483647;
  return (int)q;
}

int st_create_batch(const st_options* sets, int nsets, int device, st_ctx** out) {
  if (!out || (!sets && nsets > 0) || nsets < 1) return fail(ST_ERR_ARG, "need at least one parameter set");
  *out = nullptr;
  st_ctx* c = new st_ctx();
  c->device = device;
  int64_t first = 0;
  for (int k = 0; k < nsets; ++k) {
    SetParams P;
    int r = build_params(sets[k], first, &P);
    if (r != ST_OK) {
      delete c;
      return r;
    }
    c->opts.push_back(sets[k]);
    c->sets_h.push_back(P);
    first += sets[k].numParticles;
    if ((sets[k].integratorType == 6) != (sets[0].integratorType == 6)) {
      delete c;
      return fail(ST_ERR_UNSUPPORTED, "integratorType 6 sets cannot share a context with spin-integrating sets");
    }
  }
  c->n = first;
  c->spectrum = sets[0].integratorType == 6;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) {
    delete c;
    return fail(ST_ERR_CUDA, std::string("device setup: ") + cudaGetErrorString(e));
  }
  int r = ctx_alloc(c);
  if (r != ST_OK) {
    st_destroy(c);
    return r;
  }
  *out = c;
  return ST_OK;
}

int st_create(const st_options* opt, int device, st_ctx** out) {
  if (!opt) return fail(ST_ERR_ARG, "null options");
  return st_create_batch(opt, 1, device, out);
}

void st_destroy(st_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->arena);
  cudaFree(c->sets_d);
  cudaFree(c->status_d);
  cudaFree(c->order_d);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  cudaFree(c->ens_buf);
  cudaFree(c->spec_sets_d);
  cudaFree(c->spec_pp);
  cudaFree(c->adj_lam_buf);
  cudaFree(c->tape_pool);
  cudaFree(c->tape_prev);
  cudaFree(c->tape_pp);
  cudaFree(c->tape_head);
  cudaFree(c->tail_head);
  cudaFree(c->tape_error);
  cudaFree(c->ckpt_arena);
  cudaFree(c->replay_arena);
  if (c->status_h) cudaFreeHost(c->status_h);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int st_init(st_ctx* c) {
  if (!c) return fail(ST_ERR_ARG, "null context");
  ST_CUDA(cudaSetDevice(c->device));
  st::RunArgs a = make_args(c, 0, 0, nullptr);
  int e = st::launch_init(a, 256, c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("init launch: ") + cudaGetErrorString((cudaError_t)e));
  ST_CUDA(cudaStreamSynchronize(c->stream));
  c->initialized = true;
  c->window_grid = true;
  c->fresh = true;
  c->adj_recorded = false;
  return ST_OK;
}

int st_run_until(st_ctx* c, double next_t) {
  if (!c) return fail(ST_ERR_ARG, "null context");
  if (!c->initialized) return fail(ST_ERR_STATE, "st_run_until before st_init");
  ST_TRY(begin_run(c));
  st::RunArgs a = make_args(c, 0, 0, nullptr);
  ST_TRY(arm_deadline(c, a));
  c->fresh = false;
  c->adj_recorded = false;
  int e = c->spectrum ? st::launch_spectrum(a, -1, next_t, c->spec, c->stream)
                      : st::launch_until(a, next_t, plain_block(c), c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("plain launch: ") + cudaGetErrorString((cudaError_t)e));
  c->window_grid = false;
  return end_run(c, 1);
}

namespace {
constexpr size_t kMaxRunGraphs = 8;

// The launches of one st_run_windows call, enqueued on the context's stream.
int enqueue_run(st_ctx* c, int kernel, int w_begin, int w_end, void* snap, int* launches) {
  ST_CUDA(cudaMemsetAsync(c->status_d, 0, sizeof(st::RunStatus), c->stream));
  if (kernel == ST_KERNEL_PLAIN || c->spectrum) {  // integratorType 6 runs its own kernel, window by window
    st::RunArgs a = make_args(c, w_begin, w_end, snap);
    ST_TRY(arm_deadline(c, a));
    for (int w = w_begin; w < w_end; ++w) {
      int e = c->spectrum ? st::launch_spectrum(a, w, 0.0, c->spec, c->stream)
                          : st::launch_plain_window(a, w, plain_block(c), c->stream);
      if (e) return fail(ST_ERR_CUDA, std::string("plain launch: ") + cudaGetErrorString((cudaError_t)e));
      ++*launches;
      if (snap) {
        e = st::launch_pack_snapshot(a, w - w_begin, c->stream);
        if (e) return fail(ST_ERR_CUDA, std::string("pack launch: ") + cudaGetErrorString((cudaError_t)e));
        ++*launches;
      }
    }
    return ST_OK;
  }
  ST_TRY(run_persistent(c, w_begin, w_end, snap));
  ++*launches;
  return ST_OK;
}
}  // namespace

int st_run_windows(st_ctx* c, int kernel, int w_begin, int w_end, void* snap) {
  if (!c) return fail(ST_ERR_ARG, "null context");
  if (!c->initialized) return fail(ST_ERR_STATE, "st_run_windows before st_init");
  if (!c->window_grid) return fail(ST_ERR_STATE, "particles were advanced off the window grid by st_run_until");
  if (w_begin < 0 || w_end < w_begin) return fail(ST_ERR_ARG, "bad window range");
  if (kernel != ST_KERNEL_PLAIN && kernel != ST_KERNEL_PERSISTENT) return fail(ST_ERR_ARG, "unknown kernel selector");
  if (w_end == w_begin) return ST_OK;
  ST_CUDA(cudaSetDevice(c->device));
  if (kernel == ST_KERNEL_PERSISTENT && !c->spectrum) {  // allocations and tuning happen outside the capture
    ST_TRY(ctx_build_order(c));
    if (c->lc.variant < 0 || c->lc.blocks_per_sm <= 0) ST_TRY(autotune(c));
    if (int e = st::persistent_prepare(c->lc.variant))
      return fail(ST_ERR_CUDA, std::string("kernel attributes: ") + cudaGetErrorString((cudaError_t)e));
  }
  c->fresh = false;
  c->adj_recorded = false;
  const bool plain_shape = kernel == ST_KERNEL_PLAIN || c->spectrum;
  const int block = plain_shape ? plain_block(c) : 0;
  const int var = plain_shape ? -1 : c->lc.variant;
  const int bps = plain_shape ? 0 : c->lc.blocks_per_sm;
  size_t hit = c->graphs.size();
  for (size_t k = 0; k < c->graphs.size(); ++k) {
    const auto& g = c->graphs[k];
    if (g.kernel == kernel && g.w_begin == w_begin && g.w_end == w_end && g.snap == snap && g.block == block &&
        g.variant == var && g.bps == bps && g.deadline_s == c->deadline_s)
      hit = k;
  }
  bool captured = false;
  if (hit == c->graphs.size()) {
    int launches = 0;
    cudaGraph_t graph = nullptr;
    ST_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = enqueue_run(c, kernel, w_begin, w_end, snap, &launches);
    const cudaError_t ce = cudaStreamEndCapture(c->stream, &graph);
    if (rc != ST_OK) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (ce != cudaSuccess) return fail(ST_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) return fail(ST_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
    if (c->graphs.size() >= kMaxRunGraphs) {
      cudaGraphExecDestroy(c->graphs.front().exec);
      c->graphs.erase(c->graphs.begin());
    }
    c->graphs.push_back({kernel, w_begin, w_end, block, var, bps, snap, c->deadline_s, exec, launches});
    hit = c->graphs.size() - 1;
    captured = true;
  }
  const st_ctx::RunGraph g = c->graphs[hit];
  ST_CUDA(cudaGraphLaunch(g.exec, c->stream));
  const int rc = end_run(c, g.launches);
  c->last.graph_launches = 1;
  c->last.graph_captures = captured ? 1 : 0;
  return rc;
}

size_t st_snapshot_bytes(const st_ctx* c) { return c ? c->snap.bytes : 0; }
size_t st_snapshot_field_offset(const st_ctx* c, int f) {
  return (c && f >= 0 && f < st::kSnapFields) ? c->snap.off[f] : 0;
}

int st_read_state(st_ctx* c, const st_state_view* h) {
  if (!c || !h) return fail(ST_ERR_ARG, "null argument");
  ST_CUDA(cudaSetDevice(c->device));
  const size_t n = (size_t)c->n;
  if (n == 0) return ST_OK;
  ST_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<double> tmp(n);
  auto get = [&](const void* src, void* dst, size_t bytes) -> int {
    ST_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return ST_OK;
  };
  auto get3 = [&](double* const xs, double* const ys, double* const zs, st_vec3* dst) -> int {
    if (!dst) return ST_OK;
    ST_TRY(get(xs, tmp.data(), 8 * n));
    for (size_t i = 0; i < n; ++i) dst[i].x = tmp[i];
    ST_TRY(get(ys, tmp.data(), 8 * n));
    for (size_t i = 0; i < n; ++i) dst[i].y = tmp[i];
    ST_TRY(get(zs, tmp.data(), 8 * n));
    for (size_t i = 0; i < n; ++i) dst[i].z = tmp[i];
    return ST_OK;
  };
  if (h->t) ST_TRY(get(c->s.t, h->t, 8 * n));
  ST_TRY(get3(c->s.px, c->s.py, c->s.pz, h->pos));
  ST_TRY(get3(c->s.vx, c->s.vy, c->s.vz, h->v));
  ST_TRY(get3(c->s.Sx, c->s.Sy, c->s.Sz, h->S));
  if (h->fail) ST_TRY(get(c->s.fail, h->fail, 4 * n));
  if (h->n_coll) ST_TRY(get(c->s.n_coll, h->n_coll, 8 * n));
  if (h->n_bounce) ST_TRY(get(c->s.n_bounce, h->n_bounce, 8 * n));
  if (h->n_steps) ST_TRY(get(c->s.n_steps, h->n_steps, 8 * n));
  return ST_OK;
}

int st_gather_spins(st_ctx* c, double* dst) {
  if (!c || !dst) return fail(ST_ERR_ARG, "null argument");
  ST_CUDA(cudaSetDevice(c->device));
  if (c->n == 0) return ST_OK;
  const double* src[3] = {c->s.Sx, c->s.Sy, c->s.Sz};
  for (int k = 0; k < 3; ++k)
    ST_CUDA(cudaMemcpy2DAsync(dst + k, 3 * sizeof(double), src[k], sizeof(double), sizeof(double), (size_t)c->n,
                              cudaMemcpyDeviceToDevice, c->stream));
  ST_CUDA(cudaStreamSynchronize(c->stream));
  return ST_OK;
}

int st_gather_phase(st_ctx* c, double* dst) {
  if (!c || !dst) return fail(ST_ERR_ARG, "null argument");
  ST_CUDA(cudaSetDevice(c->device));
  int e = st::launch_gather_phase(c->s.Sy, c->s.Sz, c->s.turns, c->n, dst, c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("phase launch: ") + cudaGetErrorString((cudaError_t)e));
  ST_CUDA(cudaStreamSynchronize(c->stream));
  return ST_OK;
}

int st_device_state(st_ctx* c, st_device_soa* o) {
  if (!c || !o) return fail(ST_ERR_ARG, "null argument");
  o->n_total = c->n;
  o->t = c->s.t;
  o->pos_x = c->s.px; o->pos_y = c->s.py; o->pos_z = c->s.pz;
  o->v_x = c->s.vx; o->v_y = c->s.vy; o->v_z = c->s.vz;
  o->S_x = c->s.Sx; o->S_y = c->s.Sy; o->S_z = c->s.Sz;
  o->h = c->s.h;
  o->next_gas = c->s.next_gas;
  o->fail = c->s.fail;
  o->n_coll = c->s.n_coll; o->n_bounce = c->s.n_bounce; o->n_steps = c->s.n_steps;
  o->stop = c->s.stop;
  return ST_OK;
}

void* st_get_stream(st_ctx* c) { return c ? (void*)c->stream : nullptr; }

int st_set_params(st_ctx* c, const st_options* sets, int nsets) {
  if (!c || !sets || nsets != (int)c->sets_h.size()) return fail(ST_ERR_ARG, "st_set_params needs one options per set");
  std::vector<SetParams> P(c->sets_h.size());
  for (int k = 0; k < nsets; ++k) {
    if (sets[k].numParticles != c->opts[k].numParticles)
      return fail(ST_ERR_ARG, "st_set_params cannot change a set's particle count");
    if ((sets[k].integratorType == 6) != c->spectrum)
      return fail(ST_ERR_UNSUPPORTED, "st_set_params cannot switch between integratorType 6 and the spin integrators");
    ST_TRY(build_params(sets[k], c->sets_h[k].first, &P[k]));
  }
  std::vector<st::SpecSet> q(c->spectrum ? (size_t)nsets : 0);
  for (size_t k = 0; k < q.size(); ++k)
    if (st::build_spec_set(sets[k], &q[k]) != 0) return fail(ST_ERR_ARG, "integratorType 6: no Floquet period");
  ST_CUDA(cudaSetDevice(c->device));
  // Captured run graphs hold the kernel instantiation chosen for the old sets
  // (with or without gas collisions, integrator types 2-5) and the work order
  // grouped by their integrators: when those change, drop both.  Values
  // alone (fields, tolerances, times) are read from the device table.
  bool kernels_change = false;
  for (int k = 0; k < nsets; ++k)
    kernels_change |= P[k].gas != c->sets_h[k].gas || P[k].integrator != c->sets_h[k].integrator;
  if (kernels_change) {
    ST_CUDA(cudaStreamSynchronize(c->stream));
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    cudaFree(c->order_d);
    c->order_d = nullptr;
  }
  ST_CUDA(cudaMemcpyAsync(c->sets_d, P.data(), sizeof(SetParams) * P.size(), cudaMemcpyHostToDevice, c->stream));
  if (int e = st::launch_prepare_sets(c->sets_d, nsets, c->stream))
    return fail(ST_ERR_CUDA, std::string("prepare sets: ") + cudaGetErrorString((cudaError_t)e));
  if (!q.empty())
    ST_CUDA(cudaMemcpyAsync(c->spec_sets_d, q.data(), sizeof(st::SpecSet) * q.size(), cudaMemcpyHostToDevice,
                            c->stream));
  for (int k = 0; k < nsets; ++k) c->opts[k] = sets[k];
  c->sets_h = P;
  c->adj_recorded = false;  // a recorded tape belongs to the old parameters
  // A tuned configuration belongs to the old sets' kernels, and a chosen one
  // may have no instantiation for the new integrator types: tune again.
  if (kernels_change && c->lc.variant >= 0 &&
      (c->lc_tuned || st::persistent_max_blocks_per_sm(c->lc.variant, ctx_kind(c)) <= 0)) {
    c->lc = {0, 0, -1};
    c->lc_tuned = false;
  }
  return ST_OK;
}

size_t st_param_table_bytes(const st_ctx* c) { return c ? sizeof(SetParams) * c->sets_h.size() : 0; }

int st_synchronize(st_ctx* c) {
  if (!c) return fail(ST_ERR_ARG, "null context");
  ST_CUDA(cudaStreamSynchronize(c->stream));
  return ST_OK;
}

int st_set_launch_config(st_ctx* c, const st_launch_config* cfg) {
  if (!c) return fail(ST_ERR_ARG, "null context");
  if (!cfg) {
    c->lc = {0, 0, -1};
    return ST_OK;
  }
  if (cfg->variant >= st::persistent_variant_count()) return fail(ST_ERR_ARG, "no such kernel variant");
  if (cfg->variant >= 0 && st::persistent_max_blocks_per_sm(cfg->variant, ctx_kind(c)) <= 0)
    return fail(ST_ERR_UNSUPPORTED, "this kernel variant is not built for the context's integrator types");
  c->lc = *cfg;
  c->lc_tuned = false;
  if (c->lc.variant >= 0 && c->lc.blocks_per_sm <= 0) {
    c->lc.blocks_per_sm = std::max(1, st::persistent_max_blocks_per_sm(c->lc.variant, ctx_kind(c)));
  }
  return ST_OK;
}

int st_launch_variant_count(void) { return st::persistent_variant_count(); }
const char* st_launch_variant_name(int v) { return st::persistent_variant_name(v); }

int st_get_launch_config(const st_ctx* c, st_launch_config* cfg) {
  if (!c || !cfg) return fail(ST_ERR_ARG, "null argument");
  *cfg = c->lc;
  return ST_OK;
}

int st_set_deadline(st_ctx* c, double seconds) {
  if (!c || !(seconds >= 0.0)) return fail(ST_ERR_ARG, "bad deadline");
  c->deadline_s = seconds;
  return ST_OK;
}

int st_get_counters(const st_ctx* c, st_counters* out) {
  if (!c || !out) return fail(ST_ERR_ARG, "null argument");
  *out = c->last;
  return ST_OK;
}

// ==================================================================== adjoint
namespace {

constexpr size_t kPageBytes = sizeof(double) * st::kTapePageD;

// Pages a particle's tape needs for n steps and m segments.
int64_t adj_replay_pages(const st_ctx* c);

inline int64_t tape_pages_for(int64_t steps, int64_t segs) {
  return (steps + st::kTapeStepsPerPage - 1) / st::kTapeStepsPerPage +
         (segs + st::kTapeSegsPerPage - 1) / st::kTapeSegsPerPage;
}

// Per-particle arrays of the tape (one allocation for the context's life).
int adj_alloc_particle_arrays(st_ctx* c) {
  if (c->tape_pp) return ST_OK;
  const size_t m = (size_t)std::max<int64_t>(c->n, 1);
  // two chain sets (replays, record) of 7 arrays, then the two work orders
  const size_t chain[] = {4 * m, 4 * m, 4 * m, 4 * m, 4 * m, 8 * m, 8 * m};
  size_t total = 2 * align256(8 * m);
  for (size_t x : chain) total += 2 * align256(x);
  cudaError_t e = cudaMalloc(&c->tape_pp, total);
  if (e != cudaSuccess) return fail(ST_ERR_NOMEM, std::string("adjoint arrays: ") + cudaGetErrorString(e));
  char* p = (char*)c->tape_pp;
  auto take = [&](size_t bytes) {
    void* q = p;
    p += align256(bytes);
    return q;
  };
  for (st::TapeArgs* t : {&c->tape, &c->tail}) {
    t->step_page = (int32_t*)take(chain[0]);
    t->step_fill = (int32_t*)take(chain[1]);
    t->seg_page = (int32_t*)take(chain[2]);
    t->seg_fill = (int32_t*)take(chain[3]);
    t->complete = (int32_t*)take(chain[4]);
    t->nsteps = (int64_t*)take(chain[5]);
    t->nsegs = (int64_t*)take(chain[6]);
  }
  c->adj_order = (int64_t*)take(8 * m);
  c->adj_gorder = (int64_t*)take(8 * m);
  ST_CUDA(cudaMalloc(&c->tape_head, sizeof(unsigned long long)));
  ST_CUDA(cudaMalloc(&c->tail_head, sizeof(unsigned long long)));
  ST_CUDA(cudaMalloc(&c->tape_error, sizeof(long long) * st::kTapeErrorSlots));
  c->tape.pool_head = c->tape_head;
  c->tail.pool_head = c->tail_head;
  c->tape.error = c->tail.error = c->tape_error;
  return ST_OK;
}

// Clear the per-particle chain heads and the pool cursor of a chain set
// (c->tape: replays; c->tail: the record pass) before a tape pass.
int adj_reset_tape(st_ctx* c, const st::TapeArgs& t) {
  const size_t m = (size_t)std::max<int64_t>(c->n, 1);
  ST_CUDA(cudaMemsetAsync(t.step_page, 0xff, 4 * m, c->stream));
  ST_CUDA(cudaMemsetAsync(t.seg_page, 0xff, 4 * m, c->stream));
  ST_CUDA(cudaMemsetAsync(t.step_fill, 0, 4 * m, c->stream));
  ST_CUDA(cudaMemsetAsync(t.seg_fill, 0, 4 * m, c->stream));
  ST_CUDA(cudaMemsetAsync(t.complete, 0, 4 * m, c->stream));
  ST_CUDA(cudaMemsetAsync(t.nsteps, 0, 8 * m, c->stream));
  ST_CUDA(cudaMemsetAsync(t.nsegs, 0, 8 * m, c->stream));
  ST_CUDA(cudaMemsetAsync(t.pool_head, 0, sizeof(unsigned long long), c->stream));
  ST_CUDA(cudaMemsetAsync(c->tape_error, 0, sizeof(long long) * st::kTapeErrorSlots, c->stream));
  return ST_OK;
}
int adj_reset_replay_tape(st_ctx* c) { return adj_reset_tape(c, c->tape); }

int adj_tape_launch(st_ctx* c, const st::RunArgs& a, const st::TapeArgs& t) {
  const int per_sm = std::max(1, st::tape_record_max_blocks_per_sm(ctx_any_ext(c) ? 1 : 0));
  int e = st::launch_tape_record(a, t, c->sm_count * per_sm, c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("adjoint tape launch: ") + cudaGetErrorString((cudaError_t)e));
  return ST_OK;
}

int adj_backward_launch(st_ctx* c, const st::RunArgs& a, const st::TapeArgs& t) {
  ST_CUDA(cudaMemsetAsync(c->status_d, 0, sizeof(st::RunStatus), c->stream));
  const int magnus = ctx_any_ext(c) ? 1 : 0;  // the record pass admits types 0 or 2, one per context
  const int per_sm = std::max(1, st::adj_backward_max_blocks_per_sm(magnus));
  int e = st::launch_adj_backward(a, t, c->sm_count * per_sm, magnus, c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("adjoint backward launch: ") + cudaGetErrorString((cudaError_t)e));
  long long rep[st::kTapeErrorSlots] = {};
  ST_CUDA(cudaMemcpyAsync(rep, c->tape_error, sizeof(rep), cudaMemcpyDeviceToHost, c->stream));
  cudaError_t se = cudaStreamSynchronize(c->stream);
  if (se != cudaSuccess) return fail(ST_ERR_CUDA, std::string("adjoint backward: ") + cudaGetErrorString(se));
  if (rep[0]) {
    static const char* what[] = {"", "a particle's tape was not stored in full", "bad chain heads",
                                 "steps left after the first segment", "a segment without steps",
                                 "a page link out of range", "a segment's first step missing"};
    std::string m = "internal: the adjoint tape was inconsistent: ";
    m += (rep[0] > 0 && rep[0] < 7) ? what[rep[0]] : "?";
    m += " (particle " + std::to_string(rep[1]) + ", step page/record " + std::to_string(rep[2]) + "/" +
         std::to_string(rep[3]) + ", segment page/record " + std::to_string(rep[4]) + "/" + std::to_string(rep[5]) +
         ", tape " + std::to_string(rep[6]) + " steps " + std::to_string(rep[7]) + " segments, walked " +
         std::to_string(rep[8]) + " steps " + std::to_string(rep[9]) + " segments)";
    return fail(ST_ERR_CUDA, m);
  }
  return ST_OK;
}

// Device state view of a checkpoint slot / the replay scratch.
st::DeviceState adj_view(st_ctx* c, void* base) {
  st::DeviceState v{};
  state_layout(v, (char*)base, c->n);
  v.set = c->s.set;  // set indices are only kept in the context's own state
  return v;
}

// Work order: particles sorted by tape length, longest first, so the lanes
// that take the last particles finish together.
int adj_upload_order(st_ctx* c, const std::vector<int64_t>& ids, int64_t* dst) {
  std::vector<int64_t> o(ids);
  std::stable_sort(o.begin(), o.end(),
                   [&](int64_t x, int64_t y) { return c->adj_nsteps_h[(size_t)x] > c->adj_nsteps_h[(size_t)y]; });
  if (!o.empty())
    ST_CUDA(cudaMemcpyAsync(dst, o.data(), 8 * o.size(), cudaMemcpyHostToDevice, c->stream));
  ST_CUDA(cudaStreamSynchronize(c->stream));  // o is freed on return
  return ST_OK;
}

// The backward over the tape in the pool, once per loss of the running
// backward (each loss has its own spin adjoints and gradient block).
int adj_backward_losses(st_ctx* c, const st::RunArgs& ab, st::TapeArgs t) {
  const size_t n = (size_t)c->n;
  for (int l = 0; l < c->adj_nloss; ++l) {
    t.lam = c->adj_lam_buf + 3 * n * (size_t)l;
    t.grad = c->adj_grad_base + (size_t)st::kNumTheta * n * (size_t)l;
    ST_TRY(adj_backward_launch(c, ab, t));
  }
  return ST_OK;
}

// Replay windows up to b_hi from checkpoint slot `slot` for the particles of
// `group` (nullptr: all), writing their tape; then run the backward over
// them.  Sets *fitted = false (and runs no backward) when the tape did not fit.
int adj_replay_and_back(st_ctx* c, int slot, int b_hi, const std::vector<int64_t>* group, const st::TapeArgs& tb,
                        bool* fitted) {
  if (group) ST_TRY(adj_upload_order(c, *group, c->adj_gorder));
  ST_CUDA(cudaMemcpyAsync(c->replay_arena, (char*)c->ckpt_arena + (size_t)slot * c->arena_bytes, c->arena_bytes,
                          cudaMemcpyDeviceToDevice, c->stream));
  ST_TRY(adj_reset_replay_tape(c));
  ST_CUDA(cudaMemsetAsync(c->status_d, 0, sizeof(st::RunStatus), c->stream));
  st::RunArgs a = make_args(c, 0, b_hi, nullptr);
  a.s = adj_view(c, c->replay_arena);
  a.order = group ? c->adj_gorder : c->order_d;
  a.nitems = group ? (int64_t)group->size() : c->n;
  a.count_work = 0;
  st::TapeArgs t = tb;
  t.ckpt_every = 0;  // a replay keeps no checkpoints
  ST_TRY(adj_tape_launch(c, a, t));
  ++c->adj_stats.replays;
  // did every particle of the replay store its whole tape?
  const size_t n = (size_t)c->n;
  std::vector<int32_t> comp(std::max<size_t>(n, 1));
  ST_CUDA(cudaMemcpyAsync(comp.data(), t.complete, 4 * n, cudaMemcpyDeviceToHost, c->stream));
  cudaError_t se = cudaStreamSynchronize(c->stream);
  if (se != cudaSuccess) return fail(ST_ERR_CUDA, std::string("adjoint replay: ") + cudaGetErrorString(se));
  bool ok = true;
  const size_t cnt = group ? group->size() : n;
  for (size_t k = 0; k < cnt && ok; ++k) {
    const size_t i = group ? (size_t)(*group)[k] : k;
    if (!c->adj_stop_h[i] && !comp[i]) ok = false;
  }
  *fitted = ok;
  if (!ok) return ST_OK;
  st::RunArgs ab = make_args(c, 0, b_hi, nullptr);
  ab.order = group ? c->adj_gorder : c->adj_order;
  ab.nitems = a.nitems;
  return adj_backward_losses(c, ab, t);  // one replay serves every loss
}

// One chunk of checkpoint intervals [k_lo, k_hi), last chunk of the run first;
// split in halves, and single intervals into particle groups, while the tape
// does not fit.
int adj_chunk(st_ctx* c, int k_lo, int k_hi, const st::TapeArgs& tb) {
  const int b_hi = std::min(k_hi * c->ckpt_every, c->adj_w_run);
  bool fitted = false;
  ST_TRY(adj_replay_and_back(c, k_lo, b_hi, nullptr, tb, &fitted));
  if (fitted) return ST_OK;
  if (k_hi - k_lo > 1) {
    const int mid = (k_lo + k_hi) / 2;
    ST_TRY(adj_chunk(c, mid, k_hi, tb));
    return adj_chunk(c, k_lo, mid, tb);
  }
  // one interval whose tape does not fit: groups of particles (the replay
  // above counted each particle's records for this interval)
  const size_t n = (size_t)c->n;
  std::vector<int64_t> ns(n), ng(n);
  ST_CUDA(cudaMemcpyAsync(ns.data(), tb.nsteps, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  ST_CUDA(cudaMemcpyAsync(ng.data(), tb.nsegs, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  ST_CUDA(cudaStreamSynchronize(c->stream));
  std::vector<int64_t> group;
  int64_t used = 0;
  auto flush = [&]() -> int {
    if (group.empty()) return ST_OK;
    bool ok = false;
    ++c->adj_stats.groups;
    ST_TRY(adj_replay_and_back(c, k_lo, b_hi, &group, tb, &ok));
    if (!ok) return fail(ST_ERR_CUDA, "internal: a particle group's tape did not fit its estimate");
    group.clear();
    used = 0;
    return ST_OK;
  };
  for (size_t i = 0; i < n; ++i) {
    if (c->adj_stop_h[i]) continue;
    const int64_t need = tape_pages_for(ns[i], ng[i]);
    if (need > adj_replay_pages(c))
      return fail(ST_ERR_NOMEM, "one particle's tape over one checkpoint interval is larger than the tape pool: "
                                "raise tape_bytes or lower windows_per_checkpoint");
    if (used + need > adj_replay_pages(c)) ST_TRY(flush());
    group.push_back((int64_t)i);
    used += need;
  }
  return flush();
}

// Tape arguments over pool pages [first, first + pages) with chain set `chains`.
st::TapeArgs adj_region(st_ctx* c, const st::TapeArgs& chains, int64_t first, int64_t pages) {
  st::TapeArgs t = chains;
  t.pool = c->tape_pool + (size_t)first * st::kTapePageD;
  t.page_prev = c->tape_prev + first;
  t.pool_pages = pages;
  t.append = 0;
  t.ckpt = adj_view(c, c->ckpt_arena);
  t.ckpt_stride = (int64_t)c->arena_bytes;
  t.ckpt_every = c->ckpt_every;
  t.ckpt_count = c->ckpt_count;
  return t;
}
// Replays: the pages after the record pass's own tape.
int64_t adj_replay_pages(const st_ctx* c) { return c->tape_pages - c->adj_tail_pages; }
st::TapeArgs adj_tape_args(st_ctx* c) { return adj_region(c, c->tape, c->adj_tail_pages, adj_replay_pages(c)); }
// The record pass's own tape (all of it when it fits, else its last intervals).
st::TapeArgs adj_record_args(st_ctx* c, int64_t pages) { return adj_region(c, c->tail, 0, pages); }

// One record launch up to window w_hi (the particles continue from their own
// window counters); the chains' counts are added to the totals (an appending
// launch continues the counts it was given).
int adj_record_launch(st_ctx* c, int w_hi, const st::TapeArgs& t, std::vector<int64_t>& ns_tot,
                      std::vector<int64_t>& ng_tot) {
  ST_TRY(begin_run(c));
  st::RunArgs a = make_args(c, 0, w_hi, nullptr);
  ST_TRY(adj_tape_launch(c, a, t));
  const size_t n = (size_t)c->n;
  std::vector<int64_t> ns(std::max<size_t>(n, 1)), ng(std::max<size_t>(n, 1));
  ST_CUDA(cudaMemcpyAsync(ns.data(), t.nsteps, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  ST_CUDA(cudaMemcpyAsync(ng.data(), t.nsegs, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  ST_TRY(end_run(c, 1));
  for (size_t i = 0; i < n; ++i) {
    ns_tot[i] = t.append ? ns[i] : ns_tot[i] + ns[i];
    ng_tot[i] = t.append ? ng[i] : ng_tot[i] + ng[i];
  }
  return ST_OK;
}

}  // namespace

int st_adjoint_record(st_ctx* c, int w_end, size_t tape_bytes, int windows_per_checkpoint) {
  if (!c) return fail(ST_ERR_ARG, "null context");
  if (!c->fresh) return fail(ST_ERR_STATE, "st_adjoint_record needs a freshly initialised context (st_init)");
  if (w_end < 0) return fail(ST_ERR_ARG, "negative window count");
  if (windows_per_checkpoint < 0) return fail(ST_ERR_ARG, "negative windows_per_checkpoint");
#if !ST_GRAD_IS_LINEAR
  return fail(ST_ERR_UNSUPPORTED, "the adjoint needs the linear grad hook (ST_GRAD_IS_LINEAR)");
#endif
  int nwin_max = 0;
  for (const auto& P : c->sets_h) {
    if (P.integrator != c->sets_h[0].integrator || (P.integrator != 0 && P.integrator != 2))
      return fail(ST_ERR_UNSUPPORTED,
                  "the adjoint differentiates DOP853 or Magnus CFET8 (integratorType 0 or 2), one type per context");
    nwin_max = std::max(nwin_max, P.nwin);
  }
  ST_CUDA(cudaSetDevice(c->device));
  ST_TRY(adj_alloc_particle_arrays(c));
  const int w_run = std::min(w_end, nwin_max);
  size_t free_b = 0, total_b = 0;
  ST_CUDA(cudaMemGetInfo(&free_b, &total_b));
  // checkpoints: slot 0 holds the start state, slot k the state at window k * every
  int every = windows_per_checkpoint;
  if (every == 0) {
    const double budget = std::max(0.10 * (double)free_b, (double)c->arena_bytes);
    every = (int)std::ceil((double)std::max(w_run, 1) * (double)c->arena_bytes / budget);
    every = std::max(every, 1);
  }
  const int count = std::max(1, (w_run + every - 1) / every);
  if (count > c->ckpt_alloc) {
    cudaFree(c->ckpt_arena);
    c->ckpt_arena = nullptr;
    c->ckpt_alloc = 0;
    cudaError_t e = cudaMalloc(&c->ckpt_arena, (size_t)count * c->arena_bytes);
    if (e != cudaSuccess) return fail(ST_ERR_NOMEM, std::string("adjoint checkpoints: ") + cudaGetErrorString(e));
    c->ckpt_alloc = count;
  }
  if (!c->replay_arena) {
    cudaError_t e = cudaMalloc(&c->replay_arena, c->arena_bytes);
    if (e != cudaSuccess) return fail(ST_ERR_NOMEM, std::string("adjoint replay state: ") + cudaGetErrorString(e));
  }
  c->ckpt_every = every;
  c->ckpt_count = count;
  // tape pool
  size_t want = tape_bytes;
  if (want == 0) {
    ST_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const double cap = 0.85 * (double)free_b;
    const double guess = (double)std::max<int64_t>(c->n, 1) * 16.0 * 1048576.0 + 64.0 * 1048576.0;
    want = (size_t)std::min(cap, guess);
  }
  const int64_t pages = std::min<int64_t>((int64_t)(want / kPageBytes), INT32_MAX - 1);
  if (pages < 1) return fail(ST_ERR_ARG, "tape pool smaller than one page");
  if (pages != c->tape_pages) {
    cudaFree(c->tape_pool);
    cudaFree(c->tape_prev);
    c->tape_pool = nullptr;
    c->tape_prev = nullptr;
    c->tape_pages = 0;
    cudaError_t e = cudaMalloc(&c->tape_pool, (size_t)pages * kPageBytes);
    if (e == cudaSuccess) e = cudaMalloc(&c->tape_prev, (size_t)pages * sizeof(int32_t));
    if (e != cudaSuccess) return fail(ST_ERR_NOMEM, std::string("adjoint tape pool: ") + cudaGetErrorString(e));
    c->tape_pages = pages;
  }
  // checkpoint 0 = the start state; later slots read "nothing to run" until written
  ST_CUDA(cudaMemcpyAsync(c->ckpt_arena, c->arena, c->arena_bytes, cudaMemcpyDeviceToDevice, c->stream));
  for (int k = 1; k < count; ++k) {
    const st::DeviceState v = adj_view(c, (char*)c->ckpt_arena + (size_t)k * c->arena_bytes);
    ST_CUDA(cudaMemsetAsync(v.w_done, 0x7f, 4 * (size_t)std::max<int64_t>(c->n, 1), c->stream));
  }
  // The record pass stores its tape with its own chain set from pool page 0.
  // A run of four or more checkpoint intervals is recorded in pieces: the
  // first interval with the tape on, whose length projects the whole tape
  // (time-uniform); if that fits the pool, the rest continues the same chains;
  // if not, the middle runs with the tape off (state checkpoints only) and the
  // last intervals that fit -- the ones the backward needs first -- are stored
  // afresh, leaving the pages after them for the backward's replays.
  const size_t n = (size_t)c->n;
  c->adj_nsteps_h.assign(std::max<size_t>(n, 1), 0);
  c->adj_nsegs_h.assign(std::max<size_t>(n, 1), 0);
  c->adj_stop_h.assign(std::max<size_t>(n, 1), 0);
  c->adj_tail_from = count;
  c->adj_tail_pages = 0;
  st::TapeArgs t = adj_record_args(c, c->tape_pages);
  ST_TRY(adj_reset_tape(c, t));
  int launches = 0;
  bool tail_mode = false;
  if (count >= 4 && w_run > every) {
    ST_TRY(adj_record_launch(c, every, t, c->adj_nsteps_h, c->adj_nsegs_h));
    ++launches;
    int64_t first_pages = 0;  // pages of the first interval (each chain's last page counted whole)
    for (size_t i = 0; i < n; ++i) first_pages += tape_pages_for(c->adj_nsteps_h[i], c->adj_nsegs_h[i]);
    const double projected = (double)first_pages * (double)count;
    if (projected <= 0.9 * (double)c->tape_pages) {
      t.append = 1;  // the whole tape should fit: continue the chains
      ST_TRY(adj_record_launch(c, w_end, t, c->adj_nsteps_h, c->adj_nsegs_h));
      ++launches;
    } else {
      tail_mode = true;
      // keep room for the replay of one interval (chunks shrink to fit it), the
      // tail takes the rest but for two partly filled pages per particle
      const double reserve = 1.25 * (double)first_pages + 2.0 * (double)n;
      int keep = (int)std::floor((0.9 * (double)c->tape_pages - reserve - 2.0 * (double)n) /
                                 std::max<double>((double)first_pages, 1.0));
      keep = std::max(0, std::min(keep, count - 1));
      const int k_tail = count - keep;
      if (k_tail > 1) {  // the middle, tape off
        st::TapeArgs off = adj_record_args(c, 0);
        ST_TRY(adj_record_launch(c, std::min(k_tail * every, w_end), off, c->adj_nsteps_h, c->adj_nsegs_h));
        ++launches;
      }
      ST_TRY(adj_reset_tape(c, t));
      if (keep > 0) {
        ST_TRY(adj_record_launch(c, w_end, t, c->adj_nsteps_h, c->adj_nsegs_h));
        ++launches;
        c->adj_tail_from = k_tail;
      }
    }
  } else {
    ST_TRY(adj_record_launch(c, w_end, t, c->adj_nsteps_h, c->adj_nsegs_h));
    ++launches;
  }
  std::vector<int32_t> comp(std::max<size_t>(n, 1));
  unsigned long long head = 0;
  ST_CUDA(cudaMemcpyAsync(c->adj_stop_h.data(), c->s.stop, n, cudaMemcpyDeviceToHost, c->stream));
  ST_CUDA(cudaMemcpyAsync(comp.data(), t.complete, 4 * n, cudaMemcpyDeviceToHost, c->stream));
  ST_CUDA(cudaMemcpyAsync(&head, c->tail_head, sizeof(head), cudaMemcpyDeviceToHost, c->stream));
  ST_CUDA(cudaStreamSynchronize(c->stream));
  c->fresh = false;
  c->window_grid = true;
  bool stored = true;  // every live particle's chains of the last record launch complete
  uint64_t used = 0;
  for (size_t i = 0; i < n; ++i) {
    used += (uint64_t)tape_pages_for(c->adj_nsteps_h[i], c->adj_nsegs_h[i]) * kPageBytes;
    if (!c->adj_stop_h[i] && !comp[i]) stored = false;
  }
  const bool resident = stored && !tail_mode;
  if (tail_mode && stored && c->adj_tail_from < count) {
    c->adj_tail_pages = std::min<int64_t>((int64_t)head, c->tape_pages);
  } else {
    c->adj_tail_from = count;  // nothing kept apart from a resident tape
  }
  if (resident) c->adj_tail_pages = c->tape_pages;  // the record's chains hold all of it
  std::vector<int64_t> all(n);
  for (size_t i = 0; i < n; ++i) all[i] = (int64_t)i;
  ST_TRY(adj_upload_order(c, all, c->adj_order));
  c->adj_w_end = w_end;
  c->adj_w_run = w_run;
  c->adj_resident = resident;
  c->adj_recorded = true;
  c->adj_stats = st_adjoint_stats{};
  c->adj_stats.tape_bytes_used = used;
  c->adj_stats.tape_bytes_pool = (uint64_t)c->tape_pages * kPageBytes;
  c->adj_stats.resident = resident ? 1 : 0;
  c->adj_stats.checkpoints = count;
  c->adj_stats.windows_per_checkpoint = every;
  c->adj_stats.tail_from = c->adj_tail_from;
  c->adj_stats.record_launches = launches;
  return ST_OK;
}

int st_adjoint_backward(st_ctx* c, const double* dL_dS, double* grad, int flags) {
  return st_adjoint_backward_multi(c, 1, dL_dS, grad, flags);
}

int st_adjoint_backward_multi(st_ctx* c, int nloss, const double* dL_dS, double* grad, int flags) {
  if (!c || !dL_dS || !grad) return fail(ST_ERR_ARG, "null argument");
  if (nloss < 1) return fail(ST_ERR_ARG, "nloss must be at least 1");
  if (!c->adj_recorded) return fail(ST_ERR_STATE, "st_adjoint_backward needs st_adjoint_record first");
  ST_CUDA(cudaSetDevice(c->device));
  const size_t n = (size_t)c->n;
  c->adj_stats.replays = 0;
  c->adj_stats.groups = 0;
  if (n == 0) return ST_OK;
  const size_t lam_d = 3 * n * (size_t)nloss;
  if (lam_d > c->adj_lam_cap) {
    cudaFree(c->adj_lam_buf);
    c->adj_lam_buf = nullptr;
    c->adj_lam_cap = 0;
    cudaError_t e = cudaMalloc(&c->adj_lam_buf, sizeof(double) * lam_d);
    if (e != cudaSuccess) return fail(ST_ERR_NOMEM, std::string("adjoint spin adjoints: ") + cudaGetErrorString(e));
    c->adj_lam_cap = lam_d;
  }
  c->adj_nloss = nloss;
  c->adj_grad_base = grad;
  st::TapeArgs t = adj_tape_args(c);
  t.final_stop = c->s.stop;
  t.pulse_grads = (flags & 1) ? 1 : 0;
  ST_CUDA(cudaMemcpyAsync(c->adj_lam_buf, dL_dS, sizeof(double) * lam_d, cudaMemcpyDeviceToDevice, c->stream));
  ST_CUDA(cudaMemsetAsync(grad, 0, sizeof(double) * st::kNumTheta * n * (size_t)nloss, c->stream));
  ST_CUDA(cudaMemsetAsync(c->tape_error, 0, sizeof(long long) * st::kTapeErrorSlots, c->stream));
  if (c->adj_resident || c->adj_tail_from < c->ckpt_count) {
    // the record pass's own tape: all of it, or its last intervals
    st::TapeArgs tr = adj_record_args(c, c->adj_tail_pages);
    tr.final_stop = t.final_stop;
    tr.pulse_grads = t.pulse_grads;
    st::RunArgs a = make_args(c, 0, c->adj_w_end, nullptr);
    a.order = c->adj_order;
    a.nitems = c->n;
    ST_TRY(adj_backward_losses(c, a, tr));
    if (c->adj_resident) return ST_OK;
  }
  // replay chunks of checkpoint intervals, last first, each sized from the
  // record pass's tape length (time-uniform estimate; halves when it misses)
  int64_t total_pages = 0, live = 0;
  for (size_t i = 0; i < n; ++i) {
    if (c->adj_stop_h[i]) continue;
    total_pages += tape_pages_for(c->adj_nsteps_h[i], c->adj_nsegs_h[i]);
    ++live;
  }
  const double per_interval = (double)total_pages / (double)c->ckpt_count + 2.0 * (double)live;
  int k_hi = c->adj_tail_from;  // intervals before the kept tail
  while (k_hi > 0) {
    int span = (int)std::floor(0.85 * (double)adj_replay_pages(c) / std::max(per_interval, 1.0));
    span = std::max(1, std::min(span, k_hi));
    ST_TRY(adj_chunk(c, k_hi - span, k_hi, t));
    k_hi -= span;
  }
  return ST_OK;
}

int st_adjoint_get_stats(const st_ctx* c, st_adjoint_stats* out) {
  if (!c || !out) return fail(ST_ERR_ARG, "null argument");
  *out = c->adj_stats;
  return ST_OK;
}

int st_ensemble_stats(st_ctx* c, const void* snap, int set, st_ensemble* out) {
  if (!c || !out) return fail(ST_ERR_ARG, "null argument");
  if (set < 0 || set >= (int)c->sets_h.size()) return fail(ST_ERR_ARG, "no such parameter set");
  ST_CUDA(cudaSetDevice(c->device));
  const size_t ctl_b = 256, part_b = sizeof(double) * 8 * st::kEnsMaxBlocks;
  if (!c->ens_buf) {
    cudaError_t e = cudaMalloc(&c->ens_buf, ctl_b + part_b + sizeof(unsigned int) * st::kEnsHistBins);
    if (e != cudaSuccess) return fail(ST_ERR_NOMEM, std::string("ensemble scratch: ") + cudaGetErrorString(e));
  }
  double* ctl = (double*)c->ens_buf;
  double* part = (double*)((char*)c->ens_buf + ctl_b);
  unsigned int* hist = (unsigned int*)((char*)c->ens_buf + ctl_b + part_b);
  const double *t, *sx, *sy, *sz;
  const int32_t *fl, *tn;
  if (snap) {
    const char* b = (const char*)snap;
    t = (const double*)(b + c->snap.off[0]);
    sx = (const double*)(b + c->snap.off[7]);
    sy = (const double*)(b + c->snap.off[8]);
    sz = (const double*)(b + c->snap.off[9]);
    fl = (const int32_t*)(b + c->snap.off[10]);
    tn = (const int32_t*)(b + c->snap.off[14]);
  } else {
    t = c->s.t;
    sx = c->s.Sx;
    sy = c->s.Sy;
    sz = c->s.Sz;
    fl = c->s.fail;
    tn = c->s.turns;
  }
  const SetParams& P = c->sets_h[(size_t)set];
  int e = st::ensemble_device(t, sx, sy, sz, fl, tn, P.first, P.n, ctl, part, hist, st::kEnsMaxBlocks, c->stream);
  if (e) return fail(ST_ERR_CUDA, std::string("ensemble launch: ") + cudaGetErrorString((cudaError_t)e));
  double h[32];
  ST_CUDA(cudaMemcpyAsync(h, ctl, sizeof(double) * st::ensemble_ctl_count(), cudaMemcpyDeviceToHost, c->stream));
  cudaError_t se = cudaStreamSynchronize(c->stream);
  if (se != cudaSuccess) return fail(ST_ERR_CUDA, std::string("ensemble: ") + cudaGetErrorString(se));
  const double pi = 3.141592653589793;
  const double n = h[st::ENS_COUNT];
  st_ensemble r{};
  r.t = h[st::ENS_T];
  r.n_valid = (int64_t)n;
  r.n_phase = (int64_t)h[st::ENS_KEPT];
  for (int k = 0; k < 3; ++k) r.mean_S[k] = h[st::ENS_SX + k] / n;
  r.polarisation = std::sqrt(r.mean_S[0] * r.mean_S[0] + r.mean_S[1] * r.mean_S[1] + r.mean_S[2] * r.mean_S[2]);
  double m = h[st::ENS_MEAN2];
  if (m > pi) m -= 2.0 * pi;
  if (m < -pi) m += 2.0 * pi;
  r.phase_mean = m;
  r.phase_std = h[st::ENS_STD2];
  r.phase_stderr = r.phase_std / std::sqrt(h[st::ENS_KEPT]);
  const double b0 = std::sqrt(P.B0x * P.B0x + P.B0y * P.B0y + P.B0z * P.B0z);
  const double sgn = P.B0x > 0.0 ? 1.0 : (P.B0x < 0.0 ? -1.0 : 0.0);
  const double w = P.gamma * b0 * sgn;
  r.phase_expected = std::atan2(std::cos(w * r.t), std::sin(w * r.t));
  double shift = r.phase_mean - r.phase_expected;
  if (shift > pi) shift -= 2.0 * pi;
  if (shift < -pi) shift += 2.0 * pi;
  r.freq_shift = shift / r.t / (2.0 * pi);
  r.freq_shift_err = r.phase_stderr / r.t / (2.0 * pi);
  r.phase_unwrapped_mean = h[st::ENS_UMEAN];
  r.phase_unwrapped_std = h[st::ENS_USTD];
  const double phi0 = std::atan2(P.yi_z, P.yi_y);
  r.freq_shift_unwrapped = (r.phase_unwrapped_mean - (phi0 - w * r.t)) / r.t / (2.0 * pi);
  *out = r;
  return ST_OK;
}

int st_floquet_frequencies(const st_options* opt, double* freq, double* dt) {
  if (!opt || !freq || !dt) return fail(ST_ERR_ARG, "null argument");
  if (st::floquet_frequencies(*opt, freq, dt) != 0)
    return fail(ST_ERR_ARG, "integratorType 6 needs a nonzero pulse frequency w: its Floquet period is 2 pi / w");
  return ST_OK;
}

int st_spectrum_state(st_ctx* c, double* s1, double* s2, double* imag, int64_t* n_samples) {
  if (!c || !s1 || !s2 || !imag || !n_samples) return fail(ST_ERR_ARG, "null argument");
  if (!c->spectrum) return fail(ST_ERR_STATE, "st_spectrum_state: the context's sets are not integratorType 6");
  ST_CUDA(cudaSetDevice(c->device));
  const size_t n = (size_t)c->n, f3 = 3 * (size_t)st::kSpecFreqs;
  if (n == 0) return ST_OK;
  // device arrays are field-major ([(k * 3 + c) * n + i]); the caller's are per particle ([i][k][c])
  std::vector<double> buf(f3 * n);
  double* dst[3] = {s1, s2, imag};
  const double* src[3] = {c->spec.s1, c->spec.s2, c->spec.im};
  for (int a = 0; a < 3; ++a) {
    ST_CUDA(cudaMemcpyAsync(buf.data(), src[a], sizeof(double) * f3 * n, cudaMemcpyDeviceToHost, c->stream));
    ST_CUDA(cudaStreamSynchronize(c->stream));
    for (size_t i = 0; i < n; ++i)
      for (size_t j = 0; j < f3; ++j) dst[a][i * f3 + j] = buf[j * n + i];
  }
  ST_CUDA(cudaMemcpyAsync(n_samples, c->spec.nsamp, 8 * n, cudaMemcpyDeviceToHost, c->stream));
  ST_CUDA(cudaStreamSynchronize(c->stream));
  return ST_OK;
}

int st_covariance_spectrum(st_ctx* c, int set, double* variance, int64_t* n_samples) {
  if (!c || !variance || !n_samples) return fail(ST_ERR_ARG, "null argument");
  if (!c->spectrum) return fail(ST_ERR_STATE, "st_covariance_spectrum: the context's sets are not integratorType 6");
  if (set < 0 || set >= (int)c->sets_h.size()) return fail(ST_ERR_ARG, "no such parameter set");
  const size_t n = (size_t)c->n, F = st::kSpecFreqs;
  std::vector<double> s1(3 * F * n), s2(3 * F * n), im(3 * F * n);
  std::vector<int64_t> ns(std::max<size_t>(n, 1));
  ST_TRY(st_spectrum_state(c, s1.data(), s2.data(), im.data(), ns.data()));
  double fr[st::kSpecFreqs], dt = 0.0;
  if (st::floquet_frequencies(c->opts[(size_t)set], fr, &dt) != 0) return fail(ST_ERR_ARG, "no Floquet period");
  std::memset(variance, 0, sizeof(double) * F * 18);
  int64_t total = 0;
  const int64_t lo = c->sets_h[(size_t)set].first, hi = lo + c->sets_h[(size_t)set].n;
  for (int64_t i = lo; i < hi; ++i) {  // particle order, so the sum does not depend on the launch
    if (c->opts[(size_t)set].numParticles == 0) break;
    total += ns[(size_t)i];
    for (size_t k = 0; k < F; ++k) {
      // goertzel_stage_2 (src/floquet.cpp:40-47): c = a + i b, variance = c c^dag,
      // a = s1 - cos(w dt) s2, b = sin(w dt) s2; then the Laplace term on the
      // diagonal (SpectrumAggregator::get_covariance_spectrum, :130-145)
      const double angle = fr[k] * dt, ca = cos(angle), sa = sin(angle);
      double re[3], imc[3];
      for (int q = 0; q < 3; ++q) {
        const double x1 = s1[((size_t)i * F + k) * 3 + q], x2 = s2[((size_t)i * F + k) * 3 + q];
        re[q] = x1 - ca * x2;
        imc[q] = sa * x2;
      }
      double* m = variance + k * 18;
      for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {  // c_r conj(c_q)
          m[(r * 3 + q) * 2 + 0] += re[r] * re[q] + imc[r] * imc[q];
          m[(r * 3 + q) * 2 + 1] += imc[r] * re[q] - re[r] * imc[q];
        }
      for (int r = 0; r < 3; ++r) m[(r * 3 + r) * 2 + 1] += -im[((size_t)i * F + k) * 3 + r];
    }
  }
  *n_samples = total;
  return ST_OK;
}

int st_crmath_eval(int fn, const double* x, double* y, int64_t n) {
  if (fn < 0 || (fn > 5 && fn < 8) || fn > 11 || n < 0 || (n > 0 && (!x || !y)))
    return fail(ST_ERR_ARG, "st_crmath_eval: bad argument");
  if (int e = st::launch_crmath_eval(fn, x, y, n, nullptr))
    return fail(ST_ERR_CUDA, std::string("crmath: ") + cudaGetErrorString((cudaError_t)e));
  ST_CUDA(cudaDeviceSynchronize());
  return ST_OK;
}

int st_probe_fp64_peak(int device, double* tflops) {
  if (!tflops) return fail(ST_ERR_ARG, "null argument");
  ST_CUDA(cudaSetDevice(device));
  int sms = 0;
  ST_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
  double best = 0.0;
  for (int rep = 0; rep < 3; ++rep) {
    double sec = 0.0, flops = 0.0;
    int e = st::probe_fp64(sms, 1 << 14, &sec, &flops);
    if (e) return fail(ST_ERR_CUDA, std::string("fp64 probe: ") + cudaGetErrorString((cudaError_t)e));
    if (sec > 0.0) best = std::max(best, flops / sec * 1e-12);
  }
  *tflops = best;
  return ST_OK;
}

int st_write_header(void* file, const st_options* opt) {
  FILE* f = (FILE*)file;
  if (!f || !opt) return fail(ST_ERR_ARG, "null argument");
  st_options img = *opt;
  // zero the three padding bytes after keepStepSize so files are reproducible
  unsigned char* b = reinterpret_cast<unsigned char*>(&img);
  const size_t pad0 = offsetof(st_options, keepStepSize) + 1;
  std::memset(b + pad0, 0, offsetof(st_options, noiseAmplitudes) - pad0);
  if (std::fwrite(&img, sizeof(img), 1, f) != 1) return fail(ST_ERR_IO, "header write failed");
  return ST_OK;
}

int st_write_snapshot(void* file, int n, const st_state_view* h) {
  FILE* f = (FILE*)file;
  if (!f || !h || n < 0) return fail(ST_ERR_ARG, "bad argument");
  const size_t m = (size_t)n;
  bool ok = true;
  ok = ok && std::fwrite(h->t, 8, m, f) == m;
  ok = ok && std::fwrite(h->pos, 24, m, f) == m;
  ok = ok && std::fwrite(h->v, 24, m, f) == m;
  ok = ok && std::fwrite(h->S, 24, m, f) == m;
  ok = ok && std::fwrite(h->fail, 4, m, f) == m;
  ok = ok && std::fwrite(h->n_coll, 8, m, f) == m;
  ok = ok && std::fwrite(h->n_bounce, 8, m, f) == m;
  ok = ok && std::fwrite(h->n_steps, 8, m, f) == m;
  return ok ? ST_OK : fail(ST_ERR_IO, "snapshot write failed");
}

}  // extern "C"

// ==================================================================== driver
namespace {

struct HostSnap {
  std::vector<double> t;
  std::vector<st_vec3> pos, v, S;
  std::vector<int32_t> fail;
  std::vector<uint64_t> n_coll, n_bounce, n_steps;
  explicit HostSnap(size_t n) : t(n), pos(n), v(n), S(n), fail(n), n_coll(n), n_bounce(n), n_steps(n) {}
  st_state_view view() {
    return st_state_view{t.data(), pos.data(), v.data(), S.data(), fail.data(), n_coll.data(), n_bounce.data(),
                         n_steps.data()};
  }
};

// Unpack one device snapshot block (already copied to host memory).
void unpack_block(const st_ctx* c, const char* blk, HostSnap& hs) {
  const size_t n = (size_t)c->n;
  const double* f[10];
  for (int k = 0; k < 10; ++k) f[k] = reinterpret_cast<const double*>(blk + c->snap.off[k]);
  std::memcpy(hs.t.data(), f[0], 8 * n);
  for (size_t i = 0; i < n; ++i) {
    hs.pos[i] = {f[1][i], f[2][i], f[3][i]};
    hs.v[i] = {f[4][i], f[5][i], f[6][i]};
    hs.S[i] = {f[7][i], f[8][i], f[9][i]};
  }
  std::memcpy(hs.fail.data(), blk + c->snap.off[10], 4 * n);
  std::memcpy(hs.n_coll.data(), blk + c->snap.off[11], 8 * n);
  std::memcpy(hs.n_bounce.data(), blk + c->snap.off[12], 8 * n);
  std::memcpy(hs.n_steps.data(), blk + c->snap.off[13], 8 * n);
}

}  // namespace

extern "C" int st_main_analysis(const st_options* opt_in, const char* out_path, int device, int kernel,
                                double* run_seconds) {
  if (!opt_in || !out_path) return fail(ST_ERR_ARG, "null argument");
  {
    // createLogger (src/logger.cpp:192-204) picks HDF5 by the file extension;
    // like a reference build without HDF5, refuse such a name before any work
    std::string ext = out_path;
    const size_t dot = ext.find_last_of('.'), slash = ext.find_last_of('/');
    ext = (dot == std::string::npos || (slash != std::string::npos && dot < slash)) ? "" : ext.substr(dot);
    for (auto& ch : ext) ch = (char)std::tolower(static_cast<unsigned char>(ch));
    if (ext == ".hdf5" || ext == ".h5")
      return fail(ST_ERR_UNSUPPORTED, "HDF5 output is not built, but the output file has an hdf5 extension");
  }
  st_options opt = *opt_in;
  st_derive(&opt);
  st_ctx* c = nullptr;
  ST_TRY(st_create(&opt, device, &c));
  struct Guard {
    st_ctx* c;
    FILE* f;
    void* snap_d;
    void* snap_h;
    std::thread writer;  // writes one chunk of snapshots while the next one runs
    ~Guard() {
      if (writer.joinable()) writer.join();
      if (f) std::fclose(f);
      if (snap_d) cudaFree(snap_d);
      if (snap_h) cudaFreeHost(snap_h);
      st_destroy(c);
    }
  } g{c, nullptr, nullptr, nullptr, std::thread()};
  ST_TRY(st_init(c));
  g.f = std::fopen(out_path, "wb");
  if (!g.f) return fail(ST_ERR_IO, std::string("cannot open ") + out_path);
  ST_TRY(st_write_header(g.f, &opt));
  const size_t n = (size_t)c->n;
  HostSnap hs(n);
  st_state_view hv = hs.view();
  ST_TRY(st_read_state(c, &hv));
  ST_TRY(st_write_snapshot(g.f, (int)n, &hv));
  const int nwin = st_num_windows(&opt);
  double run = 0.0;
  if (kernel == ST_KERNEL_PLAIN) {
    for (int w = 0; w < nwin; ++w) {
      const double t0 = now_s();
      ST_TRY(st_run_windows(c, ST_KERNEL_PLAIN, w, w + 1, nullptr));
      run += now_s() - t0;
      ST_TRY(st_read_state(c, &hv));
      ST_TRY(st_write_snapshot(g.f, (int)n, &hv));
    }
  } else {
    // Windows in chunks whose snapshot blocks take at most a quarter of free
    // device memory and 2 GiB.  Two pinned host buffers: while the GPU runs
    // chunk k + 1, a writer thread unpacks and writes chunk k (in window
    // order); only the device-to-host copy of each chunk is serial.
    size_t free_b = 0, total_b = 0;
    ST_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t blk = std::max<size_t>(st_snapshot_bytes(c), 1);
    const size_t cap = std::min<size_t>(free_b / 4, (size_t)2 << 30);
    const int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)std::max(nwin, 1), cap / blk));
    ST_CUDA(cudaMalloc(&g.snap_d, blk * (size_t)chunk));
    ST_CUDA(cudaMallocHost(&g.snap_h, 2 * blk * (size_t)chunk));
    int werr = 0;  // set by the writer, read after joining it
    int slot = 0;
    for (int w = 0; w < nwin; w += chunk) {
      const int we = std::min(nwin, w + chunk);
      const double t0 = now_s();
      ST_TRY(st_run_windows(c, kernel, w, we, g.snap_d));
      run += now_s() - t0;
      // the writer that last used this buffer finished before the previous chunk was handed over
      char* hb = (char*)g.snap_h + (size_t)slot * blk * (size_t)chunk;
      ST_CUDA(cudaMemcpy(hb, g.snap_d, blk * (size_t)(we - w), cudaMemcpyDeviceToHost));
      if (g.writer.joinable()) g.writer.join();
      if (werr) return fail(ST_ERR_IO, "snapshot write failed");
      const int count = we - w;
      g.writer = std::thread([c, hb, count, blk, n, &hs, &werr, f = g.f]() {
        st_state_view v = hs.view();
        for (int k = 0; k < count && !werr; ++k) {
          unpack_block(c, hb + blk * (size_t)k, hs);
          if (st_write_snapshot(f, (int)n, &v) != ST_OK) werr = 1;
        }
      });
      slot ^= 1;
    }
    if (g.writer.joinable()) g.writer.join();
    if (werr) return fail(ST_ERR_IO, "snapshot write failed");
  }
  if (run_seconds) *run_seconds = run;
  return ST_OK;
}

// ==================================================================== autotune
namespace {

// Tuned configurations, keyed by the workload's shape, reused by every later
// context of the process.
struct TuneKey {
  int ntypes_mask;  // bit 0: a DOP853 set, bit 1: an RK45 set, bit 2: trajectory-only, bit 3 + t - 2: type t in 2-5
  int log2n;
  bool operator<(const TuneKey& o) const {
    return ntypes_mask != o.ntypes_mask ? ntypes_mask < o.ntypes_mask : log2n < o.log2n;
  }
};
// Process-wide choices, shared by contexts on any host thread.
std::map<TuneKey, st_launch_config>& tune_cache() {
  static std::map<TuneKey, st_launch_config> m;
  return m;
}
std::mutex& tune_mutex() {
  static std::mutex m;
  return m;
}

int autotune(st_ctx* c) {
  TuneKey key{0, 0};
  for (const auto& P : c->sets_h) {
    const int it = P.integrator;
    key.ntypes_mask |= it == 0 ? 1 : it == 1 ? 2 : (it >= 2 && it <= 5) ? (8 << (it - 2)) : 4;
  }
  const int ext = ctx_kind(c);
  while ((int64_t(1) << key.log2n) < c->n) ++key.log2n;
  {
    std::lock_guard<std::mutex> lock(tune_mutex());
    auto it = tune_cache().find(key);
    if (it != tune_cache().end()) {
      c->lc = it->second;
      c->lc_tuned = true;
      return ST_OK;
    }
  }
  const int nv = st::persistent_variant_count();
  // Sample: every set represented, about four particles per lane of the
  // widest candidate (one particle per lane would let the slowest particle
  // decide and favour low occupancy), one short window on a scratch context,
  // so each candidate runs for tens of milliseconds: the window is capped at
  // 50 ms of simulated time for DOP853 sets (~250 attempts per particle at
  // rtol 1e-12) and at 50 us for the fourth/fifth-order types (RK45, RKF45
  // and their quaternion forms), whose step at rtol 1e-12 is thousands of
  // times shorter.
  std::vector<st_options> sample = c->opts;
  int widest = 1;
  for (int v = 0; v < nv; ++v)
    widest = std::max(widest, st::persistent_max_blocks_per_sm(v, ext) * st::persistent_variant_block(v));
  const int64_t want = std::max<int64_t>((int64_t)c->sm_count * widest * 4, 1);
  const double frac = std::min(1.0, (double)want / (double)std::max<int64_t>(c->n, 1));
  for (auto& o : sample) {
    o.numParticles = o.numParticles > 0 ? std::max(1, (int)std::ceil(o.numParticles * frac)) : 0;
    const int it = o.integratorType;
    o.ioutInt = std::min(o.ioutInt, (it == 1 || it == 3 || it == 4 || it == 5) ? 5e-5 : 0.05);
    o.tf = o.t0 + o.ioutInt;
  }
  st_ctx* s = nullptr;
  ST_TRY(st_create_batch(sample.data(), (int)sample.size(), c->device, &s));
  double best = 1e300;
  st_launch_config best_cfg{0, 1, 1};
  // Each variant at its highest occupancy (its register budget is part of
  // the variant): on every workload measured, fewer resident blocks lost.
  for (int v = 0; v < nv; ++v) {
    if (st::persistent_max_blocks_per_sm(v, ext) <= 0) continue;  // not built for this kind of run
    // The warp-specialised and three-lane variants were slower on every
    // workload measured, and a short sample can favour them: only an explicit
    // st_set_launch_config selects them.
    if (st::persistent_variant_family(v) >= 2) continue;
    const int maxb = std::max(1, st::persistent_max_blocks_per_sm(v, ext));
    {
      st_launch_config cfg{0, maxb, v};
      st_set_launch_config(s, &cfg);
      double el = 1e300;
      for (int rep = 0; rep < 2; ++rep) {  // first repetition warms the variant up
        if (st_init(s) != ST_OK) break;
        const double t0 = now_s();
        const int r = st_run_windows(s, ST_KERNEL_PERSISTENT, 0, 1, nullptr);
        if (r == ST_OK) el = now_s() - t0;
      }
      if (el < best) {
        best = el;
        best_cfg = cfg;
      }
    }
  }
  st_destroy(s);
  c->lc = best_cfg;
  c->lc_tuned = true;
  std::lock_guard<std::mutex> lock(tune_mutex());
  tune_cache()[key] = best_cfg;
  return ST_OK;
}

}  // namespace
