// Kernel templates of the window engine (the plain, flattened and
// trajectory-ahead kernels) and their device helpers.  Included by
// st_kernels.cu (instantiations for integrator types 0 and 1) and
// st_kernels_ext.cu (EXT: also types 2-5), which compile in parallel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "st_device.cuh"

namespace st {

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Deadline armed for this run (0 = none); read once per thread.
__device__ __forceinline__ unsigned long long run_deadline(const RunArgs& a) {
  return a.deadline_armed ? *((volatile unsigned long long*)&a.status->deadline_ns) : 0ull;
}
__device__ __forceinline__ bool past_deadline(unsigned long long dl) { return dl != 0ull && globaltimer_ns() > dl; }

// Whether a set's integrator type integrates the spin in this instantiation:
// 0 DOP853, 1 RK45, and with EXT also 2-5; any other type tracks the
// trajectory only (src/particle.cpp:568-594 integrates nothing for it).
template <bool EXT>
__device__ __forceinline__ bool spin_on(int it) {
  return it == 0 || it == 1 || (EXT && it >= 2 && it <= 5);
}

// Start the integrator of the set's type over a segment.
template <bool EXT>
__device__ __forceinline__ void spin_begin(Seg& g, const SetParams& P, double Sx, double Sy, double Sz, double h) {
  if (P.integrator == 0)
    dop_begin(g, P, Sx, Sy, Sz, h);
  else if (!EXT || P.integrator == 1)
    rk45_begin(g, h);
  else
    ext_begin(g, h);
}

__device__ __forceinline__ void warp_add(unsigned long long* dst, unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}

__device__ __forceinline__ void nan_fill(PState& p) {
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  p.t = nan;
  p.px = p.py = p.pz = nan;
  p.vx = p.vy = p.vz = nan;
  p.Sx = p.Sy = p.Sz = nan;
}

__device__ __forceinline__ void write_snap(const RunArgs& a, int64_t i, int w, const PState& p) {
  if (a.snap == nullptr || w < a.w_begin || w >= a.w_end) return;
  char* b = a.snap + (size_t)(w - a.w_begin) * a.snap_layout.bytes;
  const size_t* o = a.snap_layout.off;
  reinterpret_cast<double*>(b + o[0])[i] = p.t;
  reinterpret_cast<double*>(b + o[1])[i] = p.px;
  reinterpret_cast<double*>(b + o[2])[i] = p.py;
  reinterpret_cast<double*>(b + o[3])[i] = p.pz;
  reinterpret_cast<double*>(b + o[4])[i] = p.vx;
  reinterpret_cast<double*>(b + o[5])[i] = p.vy;
  reinterpret_cast<double*>(b + o[6])[i] = p.vz;
  reinterpret_cast<double*>(b + o[7])[i] = p.Sx;
  reinterpret_cast<double*>(b + o[8])[i] = p.Sy;
  reinterpret_cast<double*>(b + o[9])[i] = p.Sz;
  reinterpret_cast<int32_t*>(b + o[10])[i] = p.fail;
  reinterpret_cast<uint64_t*>(b + o[11])[i] = p.n_coll;
  reinterpret_cast<uint64_t*>(b + o[12])[i] = p.n_bounce;
  reinterpret_cast<uint64_t*>(b + o[13])[i] = p.n_steps;
  reinterpret_cast<int32_t*>(b + o[14])[i] = p.turns;
}

// ------------------------------------------------------------------ plain
// The reference's per-particle window loop (src/particle.cpp:558-614) with
// nested segment and step loops.  Returns false if the deadline passed (the
// caller then discards the window's progress).
template <bool EXT>
__device__ __forceinline__ bool window_nested(PState& p, const SetParams& P, double tf, unsigned long long dl,
                                              unsigned long long& n_dop, unsigned long long& n_rk,
                                              unsigned long long& n_ext, unsigned long long& n_seg) {
  double tempH = p.h;
  bool finished = false;
  unsigned int guard = 0;
  while (!finished && !p.stop) {
    SegStart s0;
    finished = traj_event(p, P, tf, s0);
    ++n_seg;
    if (p.fail == 0) {
      int res = 0;
      if (spin_on<EXT>(P.integrator)) {
        Seg g;
        seg_setup(g, P, s0, p.t);
        if (P.integrator == 0) {
          dop_begin(g, P, p.Sx, p.Sy, p.Sz, tempH);
          do {
            res = dop_attempt(g, P, p.Sx, p.Sy, p.Sz);
            ++n_dop;
            if (((++guard) & 1023u) == 0u && past_deadline(dl)) return false;
          } while (res == 0);
        } else if (!EXT || P.integrator == 1) {
          rk45_begin(g, tempH);
          do {
            res = rk45_attempt(g, P, p.Sx, p.Sy, p.Sz);
            ++n_rk;
            if (((++guard) & 1023u) == 0u && past_deadline(dl)) return false;
          } while (res == 0);
        } else {
          ext_begin(g, tempH);
          do {
            res = ext_attempt(g, P, p.Sx, p.Sy, p.Sz);
            ++n_ext;
            if (((++guard) & 1023u) == 0u && past_deadline(dl)) return false;
          } while (res == 0);
        }
        tempH = g.h;
        p.turns += g.turns;
        if (res > 0) res = 0;
      }
      if (P.keep) p.h = tempH;
      if (res < 0) {
        p.stop = true;
        p.fail = res;
      }
    }
    if (p.stop) nan_fill(p);
    p.n_steps += 1;
    if (((++guard) & 255u) == 0u && past_deadline(dl)) return false;
  }
  return true;
}

// window >= 0: advance particles whose next window is `window` to its end
// ((window+1)*ioutInt of their set) and mark it done.  window < 0: advance
// every particle to next_t (runSimulation semantics, no window bookkeeping).
// EXT: also integrator types 2-5.
template <int BLOCK, bool EXT>
__global__ void __launch_bounds__(BLOCK) k_plain(RunArgs a, int window, double next_t) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long n_dop = 0, n_rk = 0, n_ext = 0, n_seg = 0;
  bool hit = false;
  const unsigned long long dl = run_deadline(a);
  if (i < a.s.n) {
    const SetParams& P = a.sets[a.s.set[i]];
    double tf = next_t;
    bool run = true;
    if (window >= 0) {
      run = window < P.nwin && a.s.w_done[i] == window;
      tf = ((double)window + 1.0) * P.ioutInt;
    }
    if (run) {
      PState p = load_state(a.s, i);
      if (window_nested<EXT>(p, P, tf, dl, n_dop, n_rk, n_ext, n_seg)) {
        store_state(a.s, i, p);
        if (window >= 0) a.s.w_done[i] = window + 1;
      } else {
        hit = true;
      }
    }
  }
  if (hit) atomicExch(&a.status->deadline_hit, 1);
  if (a.count_work) {
    warp_add(&a.status->dop_attempts, n_dop);
    warp_add(&a.status->rk45_attempts, n_rk);
    if (EXT) warp_add(&a.status->ext_attempts, n_ext);
    warp_add(&a.status->segments, n_seg);
  }
}

// ------------------------------------------------------------------ persistent
enum LaneMode { M_FETCH = 0, M_EVENT = 1, M_SEG = 2, M_WEND = 3, M_DONE = 4 };

template <int BLOCK, int MINB, bool EXT>
__global__ void __launch_bounds__(BLOCK, MINB) k_persistent(RunArgs a) {
  int mode = M_FETCH;
  int64_t i = 0;
  const SetParams* P = a.sets;
  PState p;
  Seg g;
  int w = 0, wlast = 0;
  double tf = 0.0, tempH = 0.0;
  bool finished = false, hit = false;
  unsigned long long n_dop = 0, n_rk = 0, n_ext = 0, n_seg = 0;
  unsigned int tick = 0;
  const unsigned long long dl = run_deadline(a);
  while (true) {
    // Phase A (divergent, short): bring this lane to a segment that needs
    // step attempts, or run out of work.
    while (mode != M_SEG && mode != M_DONE) {
      if (mode == M_FETCH) {
        const unsigned long long item = atomicAdd(&a.status->queue_head, 1ull);
        if (item >= (unsigned long long)a.nitems) {
          mode = M_DONE;
          break;
        }
        i = a.order ? a.order[item] : (int64_t)item;
        P = &a.sets[a.s.set[i]];
        w = a.s.w_done[i];
        wlast = min(a.w_end, P->nwin);
        if (w >= wlast) continue;
        p = load_state(a.s, i);
        tf = ((double)w + 1.0) * P->ioutInt;
        tempH = p.h;
        finished = false;
        mode = M_EVENT;
      }
      if (mode == M_EVENT) {
        if (p.stop) {
          mode = M_WEND;
        } else {
          SegStart s0;
          finished = traj_event(p, *P, tf, s0);
          ++n_seg;
          if (p.fail == 0 && spin_on<EXT>(P->integrator)) {
            seg_setup(g, *P, s0, p.t);
            spin_begin<EXT>(g, *P, p.Sx, p.Sy, p.Sz, tempH);
            mode = M_SEG;
          } else {
            if (p.fail == 0 && P->keep) p.h = tempH;
            if (p.stop) nan_fill(p);
            p.n_steps += 1;
            mode = (finished || p.stop) ? M_WEND : M_EVENT;
          }
          if (((++tick) & 255u) == 0u && past_deadline(dl)) {
            hit = true;
            mode = M_DONE;
            break;
          }
        }
      }
      if (mode == M_WEND) {
        write_snap(a, i, w, p);
        ++w;
        store_state(a.s, i, p);  // every window end is a resumable checkpoint
        a.s.w_done[i] = w;
        if (w < wlast) {
          tf = ((double)w + 1.0) * P->ioutInt;
          tempH = p.h;
          finished = false;
          mode = M_EVENT;
        } else {
          mode = M_FETCH;
        }
      }
    }
    if (mode == M_DONE) break;
    // Phase B (converged): one step attempt for every lane.
    int r;
    if (P->integrator == 0) {
      r = dop_attempt(g, *P, p.Sx, p.Sy, p.Sz);
      ++n_dop;
    } else if (!EXT || P->integrator == 1) {
      r = rk45_attempt(g, *P, p.Sx, p.Sy, p.Sz);
      ++n_rk;
    } else {
      r = ext_attempt(g, *P, p.Sx, p.Sy, p.Sz);
      ++n_ext;
    }
    if (r != 0) {
      tempH = g.h;
      p.turns += g.turns;
      if (P->keep) p.h = tempH;
      if (r < 0) {
        p.stop = true;
        p.fail = r;
      }
      if (p.stop) nan_fill(p);
      p.n_steps += 1;
      mode = (finished || p.stop) ? M_WEND : M_EVENT;
    }
    if (((++tick) & 255u) == 0u && past_deadline(dl)) {
      hit = true;
      break;
    }
  }
  if (hit) atomicExch(&a.status->deadline_hit, 1);
  if (a.count_work) {
    // lanes leave the loop at different times: aggregate with plain atomics
    if (n_dop) atomicAdd(&a.status->dop_attempts, n_dop);
    if (n_rk) atomicAdd(&a.status->rk45_attempts, n_rk);
    if (n_ext) atomicAdd(&a.status->ext_attempts, n_ext);
    if (n_seg) atomicAdd(&a.status->segments, n_seg);
  }
}

// ------------------------------------------------------------------ batched (trajectory ahead)
// The trajectory of a particle does not depend on its spin, so each lane runs
// its particle's trajectory ahead of the spin integration into a small ring of
// segment records in shared memory.  Rings are topped up warp-synchronously,
// only when many lanes have room (or one lane has run dry), so the long and
// branchy trajectory code runs with most lanes of the warp active instead of
// the few lanes whose segment just ended.  A record carries the segment's time
// span and field polynomial (o0, o1), so starting a segment on the spin side
// is a ring pop and one Bloch evaluation.  The trajectory stops at every
// window end until the spin side has finished the window, so checkpoints and
// snapshots at window ends are exact.
//
// Record fields (field-major, conflict-free): qd[(slot * kRecF + f) * BLOCK + tid]
//   f = 0 t_start, 1 t_end, 2..4 o0, 5..7 o1 (+ 8..13 p0, v0 when the grad hook is not linear)
// flags qf[slot * BLOCK + tid]: bit0 window end reached, bit1 stop, bit2 bounce, bit3 gas
// collision, bits 8-15 sanity failure code.
constexpr int kRecF = ST_GRAD_IS_LINEAR ? 8 : 14;

// ---- adjoint tape (TAPE instantiation only)
// Cursor of one particle's two tape chains.
struct TapeCursor {
  int sp, sf, gp, gf;  // step chain: last page and its records; segment chain likewise
  long long ns, ng;    // records counted (stored or not)
  bool ok;             // every record so far was stored
};

__device__ __forceinline__ void tape_open(TapeCursor& c) {
  c.sp = -1;
  c.sf = kTapeStepsPerPage;
  c.gp = -1;
  c.gf = kTapeSegsPerPage;
  c.ns = c.ng = 0;
  c.ok = true;
}

// Address of a chain's next record, or null once the pool has run out (the
// particle's tape is then incomplete and is rebuilt by a replay).
__device__ __forceinline__ double* tape_slot(const TapeArgs& t, int& page, int& fill, int per_page, int rec_d,
                                             bool& ok) {
  if (!ok) return nullptr;
  if (fill == per_page) {
    const unsigned long long np = atomicAdd(t.pool_head, 1ull);
    if (np >= (unsigned long long)t.pool_pages) {
      ok = false;
      return nullptr;
    }
    t.page_prev[np] = page;
    page = (int)np;
    fill = 0;
  }
  return t.pool + (size_t)page * kTapePageD + (size_t)(fill++) * rec_d;
}

__device__ __forceinline__ void tape_step(const TapeArgs& t, TapeCursor& c, double yx, double yy, double yz, double x,
                                          double hs) {
  ++c.ns;
  double* r = tape_slot(t, c.sp, c.sf, kTapeStepsPerPage, kTapeStepD, c.ok);
  if (r) {
    r[0] = yx; r[1] = yy; r[2] = yz; r[3] = x; r[4] = hs;
  }
}

__device__ __forceinline__ void tape_seg(const TapeArgs& t, TapeCursor& c, const SegStart& s0) {
  ++c.ng;
  double* r = tape_slot(t, c.gp, c.gf, kTapeSegsPerPage, kTapeSegD, c.ok);
  if (r) {
    r[0] = s0.t;
    r[1] = s0.px; r[2] = s0.py; r[3] = s0.pz;
    r[4] = s0.vx; r[5] = s0.vy; r[6] = s0.vz;
    r[7] = 0.0;
  }
}

// A particle's cursor at fetch: fresh chains, or (append) the chains the
// previous launch closed, continued.
__device__ __forceinline__ void tape_resume(const TapeArgs& t, TapeCursor& c, int64_t i) {
  if (!t.append) {
    tape_open(c);
    return;
  }
  c.sp = t.step_page[i];
  c.sf = c.sp < 0 ? kTapeStepsPerPage : t.step_fill[i];
  c.gp = t.seg_page[i];
  c.gf = c.gp < 0 ? kTapeSegsPerPage : t.seg_fill[i];
  c.ns = t.nsteps[i];
  c.ng = t.nsegs[i];
  c.ok = t.complete[i] != 0;
}

__device__ __forceinline__ void tape_close(const TapeArgs& t, const TapeCursor& c, int64_t i) {
  t.step_page[i] = c.sp;
  t.step_fill[i] = c.sp < 0 ? 0 : c.sf;
  t.seg_page[i] = c.gp;
  t.seg_fill[i] = c.gp < 0 ? 0 : c.gf;
  t.nsteps[i] = c.ns;
  t.nsegs[i] = c.ng;
  t.complete[i] = c.ok ? 1 : 0;
}

// View of state checkpoint k (same field layout as checkpoint 0, k * stride
// bytes on; the set indices are shared by every slot).
__device__ __forceinline__ DeviceState state_slot(const DeviceState& b, int64_t stride, int k) {
  DeviceState s = b;
  const int64_t o = stride * (int64_t)k;
#define ST_OFF(f) s.f = reinterpret_cast<decltype(s.f)>(reinterpret_cast<char*>(b.f) + o);
  ST_OFF(t) ST_OFF(px) ST_OFF(py) ST_OFF(pz) ST_OFF(vx) ST_OFF(vy) ST_OFF(vz) ST_OFF(Sx) ST_OFF(Sy) ST_OFF(Sz)
  ST_OFF(h) ST_OFF(next_gas) ST_OFF(rx) ST_OFF(ry) ST_OFF(rz) ST_OFF(rw) ST_OFF(rspare) ST_OFF(rhas) ST_OFF(fail)
  ST_OFF(n_coll) ST_OFF(n_bounce) ST_OFF(n_steps) ST_OFF(stop) ST_OFF(coll) ST_OFF(wall) ST_OFF(w_done)
  ST_OFF(turns)
#undef ST_OFF
  return s;
}

template <int BLOCK, bool TAPE, bool GAS, bool EXT>
__device__ __forceinline__ void produce_record(PState& tp, const SetParams& P, double tf, double* qd, int* qf,
                                               int slot, int tid, bool& blocked, EventDefer& dd, const TapeArgs& ta,
                                               TapeCursor& tc) {
  SegStart s0;
  const uint64_t nb = tp.n_bounce, nc = tp.n_coll;
  const bool fin = traj_event<true, GAS>(tp, P, tf, s0, &dd);
  double* r = qd + (size_t)slot * kRecF * BLOCK + tid;
  r[0 * BLOCK] = s0.t;
  r[1 * BLOCK] = tp.t;
  if (spin_on<EXT>(P.integrator)) {
    double o0[3], o1[3];
    seg_field(P, s0.px, s0.py, s0.pz, s0.vx, s0.vy, s0.vz, o0, o1);
    r[2 * BLOCK] = o0[0]; r[3 * BLOCK] = o0[1]; r[4 * BLOCK] = o0[2];
    r[5 * BLOCK] = o1[0]; r[6 * BLOCK] = o1[1]; r[7 * BLOCK] = o1[2];
#if !ST_GRAD_IS_LINEAR
    r[8 * BLOCK] = s0.px; r[9 * BLOCK] = s0.py; r[10 * BLOCK] = s0.pz;
    r[11 * BLOCK] = s0.vx; r[12 * BLOCK] = s0.vy; r[13 * BLOCK] = s0.vz;
#endif
  }
  // the segments the spin side integrates, in order
  if (TAPE && !tp.stop && tp.fail == 0) tape_seg(ta, tc, s0);
  qf[slot * BLOCK + tid] = (fin ? 1 : 0) | (tp.stop ? 2 : 0) | (tp.n_bounce != nb ? 4 : 0) |
                           (tp.n_coll != nc ? 8 : 0) | ((tp.fail & 0xff) << 8);
  if (fin || tp.stop) blocked = true;
}

enum BatchedMode { B_FETCH = 0, B_NEED = 1, B_SEG = 2, B_WEND = 3, B_DONE = 4 };

// Diffuse reflections and Maxwell-Boltzmann gas collisions are deferred
// (traj_event<true>): a lane with one pending produces no further records
// until the warp computes the pending events together (deferred_events_warp),
// when defer_k lanes have one, or one of them is about to run dry or has
// reached its window end.
// TAPE: also write the adjoint tape (steps and segments of every particle)
// and state checkpoints at every ta.ckpt_every-th window end.
// GAS = false: the instantiation for launches without gas collisions.
// STAGES = 1: DOP853 stage derivatives k2..k11 in shared memory (after the
// rings), not in registers.
// EXT: also integrator types 2-5.
template <int BLOCK, int MINB, int QCAP, bool TAPE, bool GAS, int STAGES, bool EXT>
__global__ void __launch_bounds__(BLOCK, MINB)
    k_batched(RunArgs a, int topup_start, int topup_keep, int defer_k, TapeArgs ta) {
  extern __shared__ double st_smem[];
  double* qd = st_smem;
  int* qf = reinterpret_cast<int*>(st_smem + (size_t)QCAP * kRecF * BLOCK);
  double* stage_col = st_smem + (size_t)QCAP * kRecF * BLOCK + (size_t)(QCAP * BLOCK + 1) / 2 + threadIdx.x;
  const int tid = threadIdx.x;
  const unsigned FULL = 0xffffffffu;
  int mode = B_FETCH;
  int64_t i = 0;
  const SetParams* P = a.sets;
  PState tp;  // trajectory fields run ahead; S, h, n_steps belong to the spin side
  Seg g;
  uint64_t s_ncoll = 0, s_nbounce = 0;
  int s_fail = 0;
  bool s_stop = false, cur_fin = false, blocked = true;
  int w = 0, wlast = 0, qhead = 0, qcount = 0;
  double tf = 0.0, tempH = 0.0;
  unsigned long long n_dop = 0, n_rk = 0, n_ext = 0, n_seg = 0;
  unsigned int tick = 0, dry = 0;
  bool hit = false;
  const unsigned long long dl = run_deadline(a);
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  TapeCursor tc;
  tape_open(tc);
  EventDefer dd;  // every field set: the warp's flush shuffles them from every lane
#pragma unroll
  for (int k = 0; k < 7; ++k) dd.x[k] = 0.0;
  dd.wall = 'x';
  dd.pending = false;
  dd.gas = false;
  dd.spare_first = false;
  while (true) {
    // ---- A: spin-side boundaries of this lane (pop records, window ends, fetch)
    bool starved = false;
#pragma unroll 1
    for (int guard = 0; guard < 8; ++guard) {
      if (mode == B_FETCH) {
        const unsigned long long item = atomicAdd(&a.status->queue_head, 1ull);
        if (item >= (unsigned long long)a.nitems) {
          mode = B_DONE;
          break;
        }
        i = a.order ? a.order[item] : (int64_t)item;
        P = &a.sets[a.s.set[i]];
        w = a.s.w_done[i];
        wlast = min(a.w_end, P->nwin);
        if (TAPE) tape_resume(ta, tc, i);
        dd.pending = false;
        if (w >= wlast) {
          if (TAPE) tape_close(ta, tc, i);
          continue;
        }
        tp = load_state(a.s, i);
        s_fail = tp.fail;
        s_stop = tp.stop;
        s_ncoll = tp.n_coll;
        s_nbounce = tp.n_bounce;
        qhead = qcount = 0;
        tf = ((double)w + 1.0) * P->ioutInt;
        tempH = tp.h;
        blocked = s_stop;
        mode = s_stop ? B_WEND : B_NEED;
      } else if (mode == B_NEED) {
        if (qcount == 0) {
          starved = true;
          break;
        }
        const int slot = qhead;
        qhead = (qhead + 1 == QCAP) ? 0 : qhead + 1;
        --qcount;
        const double* r = qd + (size_t)slot * kRecF * BLOCK + tid;
        const int flags = qf[slot * BLOCK + tid];
        if (flags & 4) ++s_nbounce;
        if (flags & 8) ++s_ncoll;
        cur_fin = (flags & 1) != 0;
        const int code = (int)(signed char)((flags >> 8) & 0xff);
        if (code != 0) {
          s_fail = code;
          s_stop = true;
        } else if (flags & 2) {
          s_stop = true;  // diffuse hit on an edge or corner
        }
        if (s_stop) {
          tp.Sx = tp.Sy = tp.Sz = nan;
          tp.n_steps += 1;
          mode = B_WEND;
        } else if (spin_on<EXT>(P->integrator)) {
          const double o0[3] = {r[2 * BLOCK], r[3 * BLOCK], r[4 * BLOCK]};
          const double o1[3] = {r[5 * BLOCK], r[6 * BLOCK], r[7 * BLOCK]};
          seg_begin(g, *P, r[0], r[1 * BLOCK], o0, o1);
#if !ST_GRAD_IS_LINEAR
          g.p0x = r[8 * BLOCK]; g.p0y = r[9 * BLOCK]; g.p0z = r[10 * BLOCK];
          g.v0x = r[11 * BLOCK]; g.v0y = r[12 * BLOCK]; g.v0z = r[13 * BLOCK];
#endif
          spin_begin<EXT>(g, *P, tp.Sx, tp.Sy, tp.Sz, tempH);
          mode = B_SEG;
          break;
        } else {  // trajectory only: the segment completes at once
          tp.n_steps += 1;
          if (cur_fin) mode = B_WEND;
        }
      } else if (mode == B_WEND) {
        // the window's last event reflected diffusely: its velocity is part of
        // the state, computed in phase B first (one copy of that code)
        if (dd.pending) break;
        PState out = tp;
        out.n_coll = s_ncoll;
        out.n_bounce = s_nbounce;
        out.fail = s_fail;
        out.stop = s_stop;
        if (s_stop) nan_fill(out);
        write_snap(a, i, w, out);
        ++w;
        store_state(a.s, i, out);  // every window end is a resumable checkpoint
        a.s.w_done[i] = w;
        if (TAPE && ta.ckpt_every > 0 && w % ta.ckpt_every == 0 && w / ta.ckpt_every < ta.ckpt_count) {
          const DeviceState ck = state_slot(ta.ckpt, ta.ckpt_stride, w / ta.ckpt_every);
          store_state(ck, i, out);
          ck.w_done[i] = w;
        }
        if (TAPE && w >= wlast) tape_close(ta, tc, i);
        if (w < wlast) {
          tf = ((double)w + 1.0) * P->ioutInt;
          tempH = tp.h;
          blocked = s_stop;
          mode = s_stop ? B_WEND : B_NEED;
        } else {
          mode = B_FETCH;
        }
      } else {
        break;  // B_SEG or B_DONE
      }
    }
    // ---- B: warp-synchronous trajectory top-up
    const unsigned starved_m = __ballot_sync(FULL, starved);
    const unsigned defer_m = __ballot_sync(FULL, dd.pending);
    if (defer_m != 0u &&
        (__popc(defer_m) >= defer_k || __any_sync(FULL, dd.pending && (starved || qcount <= 1 || mode == B_WEND))))
      deferred_events_warp<GAS>(tp, *P, dd, defer_m, tid & 31);
    bool prod = (mode == B_NEED || mode == B_SEG) && !blocked && qcount < QCAP && !dd.pending;
    unsigned pm = __ballot_sync(FULL, prod);
    if (starved_m != 0u || __popc(pm) >= topup_start) {
#pragma unroll 1
      for (int round = 0; round < QCAP; ++round) {
        if (prod) {
          int slot = qhead + qcount;
          if (slot >= QCAP) slot -= QCAP;
          produce_record<BLOCK, TAPE, GAS, EXT>(tp, *P, tf, qd, qf, slot, tid, blocked, dd, ta, tc);
          ++qcount;
          ++n_seg;
        }
        prod = (mode == B_NEED || mode == B_SEG) && !blocked && qcount < QCAP && !dd.pending;
        pm = __ballot_sync(FULL, prod);
        if (pm == 0u || __popc(pm) < topup_keep) break;
      }
      if (starved_m != 0u) {
        // a starved lane always gets a record in the first top-up pass; this bound only
        // protects the device from a logic error
        if (++dry > 1000000u) {
          hit = true;
          atomicExch(&a.status->pad, 1);
          break;
        }
        continue;
      }
    }
    dry = 0;
    if (__all_sync(FULL, mode == B_DONE)) break;
    // ---- C: one step attempt for every lane with an open segment
    if (mode == B_SEG) {
      int r;
      if (P->integrator == 0) {
        const double y0x = tp.Sx, y0y = tp.Sy, y0z = tp.Sz, x0 = g.x;
        if (STAGES) {
          StageSmem ks{stage_col, BLOCK};
          r = dop_attempt_ks(g, *P, tp.Sx, tp.Sy, tp.Sz, ks);
        } else {
          r = dop_attempt(g, *P, tp.Sx, tp.Sy, tp.Sz);
        }
        ++n_dop;
        if (TAPE && g.acc) tape_step(ta, tc, y0x, y0y, y0z, x0, g.hu);
      } else if (!EXT || P->integrator == 1) {
        r = rk45_attempt(g, *P, tp.Sx, tp.Sy, tp.Sz);
        ++n_rk;
      } else {
        const double y0x = tp.Sx, y0y = tp.Sy, y0z = tp.Sz, x0 = g.x;
        r = ext_attempt(g, *P, tp.Sx, tp.Sy, tp.Sz);
        ++n_ext;
        if (TAPE && g.acc) tape_step(ta, tc, y0x, y0y, y0z, x0, g.hu);
      }
      if (r != 0) {
        tempH = g.h;
        tp.turns += g.turns;
        if (P->keep) tp.h = tempH;
        if (r < 0) {
          s_fail = r;
          s_stop = true;
          qcount = 0;  // records computed past the failure are dropped
          blocked = true;
        }
        if (s_stop) tp.Sx = tp.Sy = tp.Sz = nan;
        tp.n_steps += 1;
        mode = (cur_fin || s_stop) ? B_WEND : B_NEED;
      }
    }
    if (((++tick) & 255u) == 0u && __any_sync(FULL, past_deadline(dl))) {
      hit = true;
      break;
    }
  }
  if (hit) atomicExch(&a.status->deadline_hit, 1);
  if (a.count_work) {
    warp_add(&a.status->dop_attempts, n_dop);
    warp_add(&a.status->rk45_attempts, n_rk);
    if (EXT) warp_add(&a.status->ext_attempts, n_ext);
    warp_add(&a.status->segments, n_seg);
  }
}

// ------------------------------------------------------------------ EXT instantiations
// The adjoint's record pass: the trajectory-ahead kernel with its tape on, in
// one configuration.
constexpr int kTapeBlock = 128, kTapeQcap = 6;

// Defined in st_kernels_ext.cu: the kernel of persistent variant v with
// integrator types 2-5, the record pass with them (gas-capable), and the plain
// kernel's launch with them.
const void* variant_fn_ext(int v);
const void* tape_fn_ext();
int launch_plain_ext(const RunArgs& a, int window, double next_t, int block, void* stream);

}  // namespace st
