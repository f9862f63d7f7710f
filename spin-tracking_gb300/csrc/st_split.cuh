// Warp-specialised trajectory-ahead kernel (k_split): the trajectory-ahead
// engine of k_batched with its two kinds of work on different warps.
//
// In k_batched every lane both integrates its particle's spin and, in
// warp-wide top-up passes, runs its trajectory ahead into a ring of segment
// records.  The top-up is issue- and latency-bound integer, division and
// square-root work run with the lanes that happen to need records, and while
// a warp is in it that warp issues no step attempts.  Here a block holds CW
// consumer warps and one producer warp.  A consumer lane owns one particle at
// a time and does only its spin side: it pops segment records, runs step
// attempts, writes window ends and fetches the next particle.  Each producer
// lane serves CW particle slots (slot lane + 32 c of the block): every pass it
// takes the slot of its CW whose ring holds the fewest records and runs one
// trajectory event for it, so producer lanes are busy whenever any of their
// slots has room, and the integer-heavy trajectory code overlaps the
// consumers' FP64 stream on the same SM.
//
// A slot's trajectory state lives in shared memory.  The consumer writes it at
// a particle's fetch and reads it at window ends; the producer owns it in
// between.  The handshake per slot is a single-producer single-consumer ring
// (record fields, then a block fence, then the tail counter; the consumer
// reads the record, fences, then advances the head) and a control word:
//   IDLE -> ACTIVE      consumer, after a fetch or a window end it resumed
//   ACTIVE -> BLOCKED   producer (atomicCAS), when it wrote the record that
//                       ends a window or stops the particle; it then leaves
//                       the slot alone until the consumer resumes it, so
//                       window ends stay exact, resumable checkpoints
//   ACTIVE -> STOPREQ   consumer (atomicCAS), when a step attempt failed and
//                       the particle stops: the producer may be in an event
//                       of the slot, so the consumer waits until
//   STOPREQ -> BLOCKED  producer, acknowledging between two events
//   any -> DONE         consumer, when it runs out of particles
// Waits are bounded: a consumer lane starved of records for kSplitStallNs, or
// a producer lane with work left that produced nothing for kSplitIdleNs, sets
// RunStatus::pad and the kernel winds down; the host reports that run as an
// error.  No block-wide barrier is taken after the start.
// Results equal k_batched's (and the plain kernel's) bit for bit: the producer
// runs the same trajectory event (with diffuse reflections resolved at once,
// as the plain kernel does) and the consumer the same step code.
#pragma once

#include "st_engine.cuh"

namespace st {

constexpr int kSplitIdle = 0, kSplitActive = 1, kSplitBlocked = 2, kSplitDone = 3, kSplitStopReq = 4;
constexpr int B_PARK = 5;  // consumer mode: waiting for the producer to park a stopped particle's slot
constexpr unsigned long long kSplitStallNs = 4000000000ull;  // a consumer lane starved this long: logic error
constexpr unsigned long long kSplitIdleNs = 20000000000ull;  // a producer lane idle this long with work left
// per-slot fields in shared memory (field-major over the block's slots)
enum { SD_T = 0, SD_PX, SD_PY, SD_PZ, SD_VX, SD_VY, SD_VZ, SD_NG, SD_SPARE, SD_TF, SD_N };
enum { SU_RX = 0, SU_RY, SU_RZ, SU_RW, SU_NCOLL, SU_NBOUNCE, SU_N };
enum { SI_CTL = 0, SI_HEAD, SI_TAIL, SI_FAIL, SI_SET, SI_FLAGS, SI_N };

__host__ __device__ constexpr size_t split_smem_bytes(int cw, int qcap) {
  return (size_t)cw * 32 * (8 * ((size_t)qcap * kRecF + SD_N + SU_N) + 4 * ((size_t)qcap + SI_N));
}

struct SplitSmem {
  double* qd;    // [q][field][slot] segment records
  double* sd;    // [field][slot] trajectory doubles
  uint64_t* su;  // [field][slot] RNG words and event counters
  int* qf;       // [q][slot] record flags (as k_batched's)
  int* si;       // [field][slot] control, head, tail, failure, set, packed flags
  int ns;        // slots of the block
};

__device__ __forceinline__ SplitSmem split_carve(double* base, int ns, int qcap) {
  SplitSmem m;
  m.ns = ns;
  m.qd = base;
  m.sd = m.qd + (size_t)qcap * kRecF * ns;
  m.su = reinterpret_cast<uint64_t*>(m.sd + (size_t)SD_N * ns);
  m.qf = reinterpret_cast<int*>(m.su + (size_t)SU_N * ns);
  m.si = m.qf + (size_t)qcap * ns;
  return m;
}

// The trajectory part of a particle state, to and from its slot.
__device__ __forceinline__ void slot_store(const SplitSmem& m, int j, const PState& p) {
  const int n = m.ns;
  m.sd[SD_T * n + j] = p.t;
  m.sd[SD_PX * n + j] = p.px; m.sd[SD_PY * n + j] = p.py; m.sd[SD_PZ * n + j] = p.pz;
  m.sd[SD_VX * n + j] = p.vx; m.sd[SD_VY * n + j] = p.vy; m.sd[SD_VZ * n + j] = p.vz;
  m.sd[SD_NG * n + j] = p.next_gas;
  m.sd[SD_SPARE * n + j] = p.rng.spare;
  m.su[SU_RX * n + j] = p.rng.x; m.su[SU_RY * n + j] = p.rng.y;
  m.su[SU_RZ * n + j] = p.rng.z; m.su[SU_RW * n + j] = p.rng.w;
  m.su[SU_NCOLL * n + j] = p.n_coll; m.su[SU_NBOUNCE * n + j] = p.n_bounce;
  m.si[SI_FAIL * n + j] = p.fail;
  m.si[SI_FLAGS * n + j] = (p.rng.has ? 1 : 0) | (p.stop ? 2 : 0) | ((int)(unsigned char)p.coll << 8) |
                           ((int)(unsigned char)p.wall << 16);
}
__device__ __forceinline__ void slot_load(const SplitSmem& m, int j, PState& p) {
  const int n = m.ns;
  p.t = m.sd[SD_T * n + j];
  p.px = m.sd[SD_PX * n + j]; p.py = m.sd[SD_PY * n + j]; p.pz = m.sd[SD_PZ * n + j];
  p.vx = m.sd[SD_VX * n + j]; p.vy = m.sd[SD_VY * n + j]; p.vz = m.sd[SD_VZ * n + j];
  p.next_gas = m.sd[SD_NG * n + j];
  p.rng.spare = m.sd[SD_SPARE * n + j];
  p.rng.x = m.su[SU_RX * n + j]; p.rng.y = m.su[SU_RY * n + j];
  p.rng.z = m.su[SU_RZ * n + j]; p.rng.w = m.su[SU_RW * n + j];
  p.n_coll = m.su[SU_NCOLL * n + j]; p.n_bounce = m.su[SU_NBOUNCE * n + j];
  p.fail = m.si[SI_FAIL * n + j];
  const int f = m.si[SI_FLAGS * n + j];
  p.rng.has = (f & 1) != 0;
  p.stop = (f & 2) != 0;
  p.coll = (char)((f >> 8) & 0xff);
  p.wall = (char)((f >> 16) & 0xff);
}

__device__ __forceinline__ int vload(const int* p) { return *reinterpret_cast<const volatile int*>(p); }
__device__ __forceinline__ void vstore(int* p, int v) { *reinterpret_cast<volatile int*>(p) = v; }

// One trajectory event of slot j into ring entry q (k_batched's record format).
template <bool GAS, bool EXT>
__device__ __forceinline__ void split_produce(const SplitSmem& m, int j, int q, const SetParams& P, double tf) {
  PState tp;
  slot_load(m, j, tp);
  SegStart s0;
  const uint64_t nb = tp.n_bounce, nc = tp.n_coll;
  const bool fin = traj_event<false, GAS>(tp, P, tf, s0);
  const int n = m.ns;
  double* r = m.qd + (size_t)q * kRecF * n + j;
  r[0 * n] = s0.t;
  r[1 * n] = tp.t;
  if (spin_on<EXT>(P.integrator)) {
    double o0[3], o1[3];
    seg_field(P, s0.px, s0.py, s0.pz, s0.vx, s0.vy, s0.vz, o0, o1);
    r[2 * n] = o0[0]; r[3 * n] = o0[1]; r[4 * n] = o0[2];
    r[5 * n] = o1[0]; r[6 * n] = o1[1]; r[7 * n] = o1[2];
#if !ST_GRAD_IS_LINEAR
    r[8 * n] = s0.px; r[9 * n] = s0.py; r[10 * n] = s0.pz;
    r[11 * n] = s0.vx; r[12 * n] = s0.vy; r[13 * n] = s0.vz;
#endif
  }
  m.qf[q * n + j] = (fin ? 1 : 0) | (tp.stop ? 2 : 0) | (tp.n_bounce != nb ? 4 : 0) | (tp.n_coll != nc ? 8 : 0) |
                    ((tp.fail & 0xff) << 8);
  slot_store(m, j, tp);
  __threadfence_block();
  // the record that ends a window or the particle parks the slot until its
  // consumer resumes it (a consumer that gave the slot up keeps it DONE)
  if (fin || tp.stop) atomicCAS(&m.si[SI_CTL * n + j], kSplitActive, kSplitBlocked);
  __threadfence_block();
  vstore(&m.si[SI_TAIL * n + j], vload(&m.si[SI_TAIL * n + j]) + 1);
}

// CW consumer warps, then PW producer warps (each producer lane serving
// CW / PW slots: lane l of the producers serves slots l + 32 PW c).  CREG,
// PREG > 0: the warpgroups' register shares after a setmaxnreg split (the
// consumers' steps want more registers than the launch gives every thread, the
// producers' trajectory events fewer); the host checks the shares against the
// registers the block is launched with before any launch.
template <int CW, int PW, int MINB, int QCAP, bool GAS, int CREG, int PREG>
__global__ void __launch_bounds__((CW + PW) * 32, MINB) k_split(RunArgs a) {
  static_assert(CW % PW == 0, "every producer lane serves the same number of slots");
  static_assert(CREG == 0 || (CW % 4 == 0 && PW % 4 == 0), "register shares are per warpgroup");
  extern __shared__ double st_smem[];
  constexpr int NS = CW * 32;
  const SplitSmem m = split_carve(st_smem, NS, QCAP);
  const unsigned FULL = 0xffffffffu;
  const int warp = threadIdx.x >> 5;
  if (warp < CW) {  // every slot starts idle with an empty ring
    const int j = threadIdx.x;
    m.si[SI_CTL * NS + j] = kSplitIdle;
    m.si[SI_HEAD * NS + j] = 0;
    m.si[SI_TAIL * NS + j] = 0;
  }
  __syncthreads();
  bool stuck = false;
  if (warp >= CW) {
    // ---------------------------------------------------------------- producers
    if (CREG > 0) asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;\n" ::"n"(PREG));
    const int pl = threadIdx.x - CW * 32;  // producer lane index
    unsigned long long n_seg = 0, idle_since = 0;
    unsigned int tick = 0;
    while (true) {
      int best = -1, best_fill = QCAP, open = 0;
#pragma unroll
      for (int c = 0; c < CW / PW; ++c) {
        const int j = pl + 32 * PW * c;
        int ctl = vload(&m.si[SI_CTL * NS + j]);
        if (ctl == kSplitStopReq) {  // no event of this slot is in flight: park it
          atomicCAS(&m.si[SI_CTL * NS + j], kSplitStopReq, kSplitBlocked);
          ctl = kSplitBlocked;
        }
        if (ctl != kSplitDone) ++open;
        if (ctl == kSplitActive) {
          const int fill = vload(&m.si[SI_TAIL * NS + j]) - vload(&m.si[SI_HEAD * NS + j]);
          if (fill < best_fill) {
            best_fill = fill;
            best = j;
          }
        }
      }
      if (!__any_sync(FULL, open > 0)) break;
      if (best >= 0) {
        __threadfence_block();  // the slot's fields as its consumer left them
        const SetParams& P = a.sets[m.si[SI_SET * NS + best]];
        const int q = vload(&m.si[SI_TAIL * NS + best]) % QCAP;
        split_produce<GAS, false>(m, best, q, P, m.sd[SD_TF * NS + best]);
        ++n_seg;
        idle_since = 0;
      } else if (open > 0) {
        const unsigned long long now = globaltimer_ns();
        if (idle_since == 0) idle_since = now;
        else if (now - idle_since > kSplitIdleNs) stuck = true;
        __nanosleep(64);
      }
      if (((++tick) & 63u) == 0u && __any_sync(FULL, stuck)) break;
    }
    if (stuck) atomicExch(&a.status->pad, 1);
    if (a.count_work) warp_add(&a.status->segments, n_seg);
    return;
  }
  // ---------------------------------------------------------------- consumers
  if (CREG > 0) asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;\n" ::"n"(CREG));
  const int j = threadIdx.x;  // this lane's slot
  int mode = B_FETCH;
  int64_t i = 0;
  const SetParams* P = a.sets;
  PState tp;  // the spin side's fields (S, h, n_steps, turns) and, at window ends, the slot's trajectory
  Seg g;
  uint64_t s_ncoll = 0, s_nbounce = 0;
  int s_fail = 0, head = 0;
  bool s_stop = false, cur_fin = false;
  int w = 0, wlast = 0;
  double tempH = 0.0;
  unsigned long long n_dop = 0, n_rk = 0, starved_since = 0;
  unsigned int tick = 0;
  bool hit = false;
  const unsigned long long dl = run_deadline(a);
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  while (true) {
    bool starved = false;
#pragma unroll 1
    for (int guard = 0; guard < 8; ++guard) {
      if (mode == B_FETCH) {
        const unsigned long long item = atomicAdd(&a.status->queue_head, 1ull);
        if (item >= (unsigned long long)a.nitems) {
          mode = B_DONE;
          atomicExch(&m.si[SI_CTL * NS + j], kSplitDone);
          break;
        }
        i = a.order ? a.order[item] : (int64_t)item;
        P = &a.sets[a.s.set[i]];
        w = a.s.w_done[i];
        wlast = min(a.w_end, P->nwin);
        if (w >= wlast) continue;
        tp = load_state(a.s, i);
        s_fail = tp.fail;
        s_stop = tp.stop;
        s_ncoll = tp.n_coll;
        s_nbounce = tp.n_bounce;
        tempH = tp.h;
        // the slot is IDLE or BLOCKED: its producer lane does not touch it
        slot_store(m, j, tp);
        m.sd[SD_TF * NS + j] = ((double)w + 1.0) * P->ioutInt;
        m.si[SI_SET * NS + j] = a.s.set[i];
        vstore(&m.si[SI_HEAD * NS + j], 0);
        vstore(&m.si[SI_TAIL * NS + j], 0);
        head = 0;
        if (s_stop) {
          mode = B_WEND;
        } else {
          __threadfence_block();
          atomicExch(&m.si[SI_CTL * NS + j], kSplitActive);
          mode = B_NEED;
        }
      } else if (mode == B_NEED) {
        if (vload(&m.si[SI_TAIL * NS + j]) == head) {
          starved = true;
          break;
        }
        __threadfence_block();
        const int q = head % QCAP;
        const double* r = m.qd + (size_t)q * kRecF * NS + j;
        const int flags = m.qf[q * NS + j];
        const double r0 = r[0], r1 = r[1 * NS];
        const double o0[3] = {r[2 * NS], r[3 * NS], r[4 * NS]};
        const double o1[3] = {r[5 * NS], r[6 * NS], r[7 * NS]};
#if !ST_GRAD_IS_LINEAR
        const double pv[6] = {r[8 * NS], r[9 * NS], r[10 * NS], r[11 * NS], r[12 * NS], r[13 * NS]};
#endif
        __threadfence_block();
        vstore(&m.si[SI_HEAD * NS + j], ++head);  // the entry is free again
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
        } else if (spin_on<false>(P->integrator)) {
          seg_begin(g, *P, r0, r1, o0, o1);
#if !ST_GRAD_IS_LINEAR
          g.p0x = pv[0]; g.p0y = pv[1]; g.p0z = pv[2];
          g.v0x = pv[3]; g.v0y = pv[4]; g.v0z = pv[5];
#endif
          spin_begin<false>(g, *P, tp.Sx, tp.Sy, tp.Sz, tempH);
          mode = B_SEG;
          break;
        } else {  // trajectory only: the segment completes at once
          tp.n_steps += 1;
          if (cur_fin) mode = B_WEND;
        }
      } else if (mode == B_WEND) {
        // the window's last record is in: the producer has parked the slot,
        // whose trajectory fields are the state at the window end
        PState out = tp;
        slot_load(m, j, out);
        out.Sx = tp.Sx; out.Sy = tp.Sy; out.Sz = tp.Sz;
        out.h = tp.h;
        out.n_steps = tp.n_steps;
        out.turns = tp.turns;
        out.n_coll = s_ncoll;
        out.n_bounce = s_nbounce;
        out.fail = s_fail;
        out.stop = s_stop;
        if (s_stop) nan_fill(out);
        write_snap(a, i, w, out);
        ++w;
        store_state(a.s, i, out);  // every window end is a resumable checkpoint
        a.s.w_done[i] = w;
        if (w < wlast) {
          m.sd[SD_TF * NS + j] = ((double)w + 1.0) * P->ioutInt;
          tempH = tp.h;
          if (s_stop) {
            mode = B_WEND;
          } else {
            __threadfence_block();
            atomicExch(&m.si[SI_CTL * NS + j], kSplitActive);
            mode = B_NEED;
          }
        } else {
          mode = B_FETCH;
        }
      } else if (mode == B_PARK) {
        if (vload(&m.si[SI_CTL * NS + j]) != kSplitBlocked) {
          starved = true;
          break;
        }
        mode = B_WEND;
      } else {
        break;  // B_SEG or B_DONE
      }
    }
    if (__all_sync(FULL, mode == B_DONE)) break;
    // one step attempt for every lane with an open segment
    if (mode == B_SEG) {
      int r;
      if (P->integrator == 0) {
        r = dop_attempt(g, *P, tp.Sx, tp.Sy, tp.Sz);
        ++n_dop;
      } else {
        r = rk45_attempt(g, *P, tp.Sx, tp.Sy, tp.Sz);
        ++n_rk;
      }
      if (r != 0) {
        tempH = g.h;
        tp.turns += g.turns;
        if (P->keep) tp.h = tempH;
        bool park = false;
        if (r < 0) {
          // the particle stops: records produced past the failure are dropped
          // with the slot's ring when the next fetch resets it; until the
          // producer has parked the slot its fields may still change
          s_fail = r;
          s_stop = true;
          park = atomicCAS(&m.si[SI_CTL * NS + j], kSplitActive, kSplitStopReq) == kSplitActive;
        }
        if (s_stop) tp.Sx = tp.Sy = tp.Sz = nan;
        tp.n_steps += 1;
        mode = park ? B_PARK : ((cur_fin || s_stop) ? B_WEND : B_NEED);
      }
    }
    if (!__any_sync(FULL, mode == B_SEG)) __nanosleep(100);  // nothing to integrate: leave the issue slots
    if (starved) {
      const unsigned long long now = globaltimer_ns();
      if (starved_since == 0) starved_since = now;
      else if (now - starved_since > kSplitStallNs) stuck = true;
    } else {
      starved_since = 0;
    }
    if (((++tick) & 255u) == 0u) {
      if (__any_sync(FULL, stuck)) break;
      if (__any_sync(FULL, past_deadline(dl))) {
        hit = true;
        break;
      }
    }
  }
  if (mode != B_DONE) atomicExch(&m.si[SI_CTL * NS + j], kSplitDone);  // let the producer wind down
  if (stuck) atomicExch(&a.status->pad, 1);
  if (hit) atomicExch(&a.status->deadline_hit, 1);
  if (a.count_work) {
    warp_add(&a.status->dop_attempts, n_dop);
    warp_add(&a.status->rk45_attempts, n_rk);
  }
}

}  // namespace st
