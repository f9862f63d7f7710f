// Three lanes per particle (k_tpp3): the threads-per-particle axis of the
// launch variants.  Lanes 3g, 3g+1, 3g+2 of a warp share particle g (ten per
// warp; lanes 30 and 31 idle).  The three run the trajectory, the window
// bookkeeping and the step controller together (the same instructions on the
// same values), and split the DOP853 stage arithmetic by spin component:
// lane 3g + c keeps only component c of the stage derivatives (12 doubles
// instead of 36), and the cross products, the error norms and the turn counter
// gather the other two components by shuffles within the group.  Every
// component is computed with the single-lane kernel's expression, and sums
// over components take the same order, so results are bit-identical to the
// other variants.  For DOP853 runs only: the host offers these variants to no
// run with RK45 sets.
// Flattened loop shape (k_persistent): a group fetches a particle, runs its
// events inline and attempts steps when its segment is open.
#pragma once

#include "st_engine.cuh"

namespace st {

struct Group3 {
  unsigned mask;  // the group's three lanes
  int base;       // its first lane
  int c;          // this lane's component
};

__device__ __forceinline__ double g3_get(const Group3& G, double v, int comp) {
  return __shfl_sync(G.mask, v, G.base + comp);
}

// f_c of f = y x O from the group's components (bloch's expression for c).
__device__ __forceinline__ double g3_cross(const Group3& G, double y, double o) {
  const int c1 = G.c == 2 ? 0 : G.c + 1, c2 = G.c == 0 ? 2 : G.c - 1;
  const double y1 = g3_get(G, y, c1), y2 = g3_get(G, y, c2);
  const double o1 = g3_get(G, o, c1), o2 = g3_get(G, o, c2);
  return fma(y1, o2, -y2 * o1);
}

__device__ __forceinline__ double pick3(int c, double x, double y, double z) { return c == 0 ? x : (c == 1 ? y : z); }

// dop_attempt_ks for component G.c: Sc, kc are this lane's components of the
// spin and of the FSAL derivative; the controller state in g is the group's.
__device__ __forceinline__ int dop_attempt_g3(const Group3& G, Seg& g, const SetParams& P, double& Sc, double& kc) {
  using namespace dop;
  const int c = G.c;
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
  const double S0 = Sc;
  // this component of the field polynomial, scaled by h (hpoly_of)
  const double q0 = h * pick3(c, g.o0x, g.o0y, g.o0z), q1 = h * pick3(c, g.o1x, g.o1y, g.o1z),
               q2 = h * pick3(c, g.o2x, g.o2y, g.o2z), qa = h * g.gpa;
  const double k1 = h * kc;
  double ks[13];
#pragma unroll
  for (int s = 2; s <= 11; ++s) {
    double acc = fma(dopst::a(s, 0), k1, S0);
#pragma unroll
    for (int j = 1; j < dopst::cnt(s); ++j) acc = fma(dopst::a(s, j), ks[dopst::src(s, j)], acc);
    const double tau = fma(dopst::c(s), h, tx);
    double O = fma(fma(q2, tau, q1), tau, q0);
    if (c == 2 && g.gpa != 0.0) O = fma(qa, cos(P.w * (g.t0 + tau)), O);
    ks[s] = g3_cross(G, acc, O);
  }
  double acc12 = fma(dopst::a(12, 0), k1, S0);
#pragma unroll
  for (int j = 1; j < dopst::cnt(12); ++j) acc12 = fma(dopst::a(12, j), ks[dopst::src(12, j)], acc12);
  const double tph = tx + h;
  double O12 = fma(fma(pick3(c, g.o2x, g.o2y, g.o2z), tph, pick3(c, g.o1x, g.o1y, g.o1z)), tph,
                   pick3(c, g.o0x, g.o0y, g.o0z));
  if (c == 2 && g.gpa != 0.0) O12 = fma(g.gpa, cos(P.w * (g.t0 + tph)), O12);
  const double k12 = g3_cross(G, acc12, h * O12);
  double acc = B1 * k1;
  acc = fma(B6, ks[6], acc);
  acc = fma(B7, ks[7], acc);
  acc = fma(B8, ks[8], acc);
  acc = fma(B9, ks[9], acc);
  acc = fma(B10, ks[10], acc);
  acc = fma(B11, ks[11], acc);
  const double bc = fma(B12, k12, acc);
  const double nc = Sc + bc;
  const double e1 = fma(-BHH3, k12, fma(-BHH2, ks[9], fma(-BHH1, k1, bc)));
  double er = ER1 * k1;
  er = fma(ER6, ks[6], er);
  er = fma(ER7, ks[7], er);
  er = fma(ER8, ks[8], er);
  er = fma(ER9, ks[9], er);
  er = fma(ER10, ks[10], er);
  er = fma(ER11, ks[11], er);
  er = fma(ER12, k12, er);
  const double wc = rcp_full(fma(P.rtol, max_d(fabs(Sc), fabs(nc)), P.atol));
  const double q1c = e1 * wc, q2c = er * wc;
  const double q1x = g3_get(G, q1c, 0), q1y = g3_get(G, q1c, 1), q1z = g3_get(G, q1c, 2);
  const double q2x = g3_get(G, q2c, 0), q2y = g3_get(G, q2c, 1), q2z = g3_get(G, q2c, 2);
  const double err2 = fma(q1z, q1z, fma(q1y, q1y, q1x * q1x));
  double err = fma(q2z, q2z, fma(q2y, q2y, q2x * q2x));
  double deno = fma(0.01, err2, err);
  if (deno <= 0.0) deno = 1.0;
  err = err * rsqrt_full(deno * 3.0);
  double hnew;
  const bool fast = (P.beta == 0.0) && (err > 1e-300) && (err < 1e300);
  double rr = 0.0, fac11 = 0.0;
  if (fast) {
    rr = rroot8(err);
    hnew = h * min_d(P.fac2, max_d(P.fac1, P.safe * rr));
  } else {
    fac11 = pow(err, P.expo1);
    double fac = fac11 / pow(g.facold, P.beta);
    fac = max_d(P.facc2, min_d(P.facc1, fac / P.safe));
    hnew = h / fac;
  }
  const double sy0 = g3_get(G, S0, 1), sz0 = g3_get(G, S0, 2);
  const double ny = g3_get(G, nc, 1), nz = g3_get(G, nc, 2);
  const double kn = g3_cross(G, nc, O12);  // FSAL: f(x + h, y_new), used if accepted
  if (err <= 1.0 || P.fixed) {
    g.acc = true;
    g.hu = h;
    g.facold = max_d(err, 1.0e-4);
    kc = kn;
    g.turns += count_turn(sy0, sz0, ny, nz);
    Sc = nc;
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
  return 0;
}

template <int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) k_tpp3(RunArgs a) {
  const int lane = threadIdx.x & 31;
  Group3 G;
  G.base = (lane / 3) * 3;
  G.c = lane - G.base;
  G.mask = 7u << G.base;
  const bool lead = G.c == 0;
  int mode = lane < 30 ? M_FETCH : M_DONE;
  int64_t i = 0;
  const SetParams* P = a.sets;
  PState p;
  Seg g;
  double Sc = 0.0, kc = 0.0;
  int w = 0, wlast = 0;
  double tf = 0.0, tempH = 0.0;
  bool finished = false, hit = false;
  unsigned long long n_dop = 0, n_seg = 0;
  unsigned int tick = 0;
  const unsigned long long dl = run_deadline(a);
  while (mode != M_DONE) {
    // the group's boundaries (the three lanes take the same path)
    while (mode != M_SEG && mode != M_DONE) {
      if (mode == M_FETCH) {
        unsigned long long item = 0;
        if (lead) item = atomicAdd(&a.status->queue_head, 1ull);
        item = __shfl_sync(G.mask, item, G.base);
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
          if (lead) ++n_seg;
          if (p.fail == 0 && spin_on<false>(P->integrator)) {
            seg_setup(g, *P, s0, p.t);
            spin_begin<false>(g, *P, p.Sx, p.Sy, p.Sz, tempH);
            Sc = pick3(G.c, p.Sx, p.Sy, p.Sz);
            kc = pick3(G.c, g.kx, g.ky, g.kz);
            mode = M_SEG;
          } else {
            if (p.fail == 0 && P->keep) p.h = tempH;
            if (p.stop) nan_fill(p);
            p.n_steps += 1;
            mode = (finished || p.stop) ? M_WEND : M_EVENT;
          }
          bool late = ((++tick) & 255u) == 0u && past_deadline(dl);
          late = __shfl_sync(G.mask, late, G.base);  // one decision per group
          if (late) {
            hit = true;
            mode = M_DONE;
            break;
          }
        }
      }
      if (mode == M_WEND) {
        if (lead) {
          write_snap(a, i, w, p);
          store_state(a.s, i, p);  // every window end is a resumable checkpoint
          a.s.w_done[i] = w + 1;
        }
        ++w;
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
    // one step attempt of the group's open segment
    int r;
    if (P->integrator == 0) {
      r = dop_attempt_g3(G, g, *P, Sc, kc);
      if (lead) ++n_dop;
      p.Sx = g3_get(G, Sc, 0);
      p.Sy = g3_get(G, Sc, 1);
      p.Sz = g3_get(G, Sc, 2);
    } else {
      // runs with RK45 sets do not get this kernel (the host leaves these
      // variants out for them); if one did, its particles stop with an error
      if (lead) atomicExch(&a.status->pad, 1);
      r = -1;
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
    bool late = ((++tick) & 255u) == 0u && past_deadline(dl);
    late = __shfl_sync(G.mask, late, G.base);
    if (late) {
      hit = true;
      break;
    }
  }
  if (hit && lead) atomicExch(&a.status->deadline_hit, 1);
  if (a.count_work) {
    if (n_dop) atomicAdd(&a.status->dop_attempts, n_dop);
    if (n_seg) atomicAdd(&a.status->segments, n_seg);
  }
}

}  // namespace st
