// Discrete adjoint of the DOP853 spin integration along the particles' fixed
// trajectories: gradients of a loss L(S_final) with respect to the field
// parameters theta = [Gx(3), Gy(3), Gz(3), B0(3), E(3), a, w].
//
// The trajectory does not depend on theta, and with the accepted step
// sequence held fixed every DOP853 step is a linear map of the spin, so the
// gradient is the exact derivative of the discrete forward map (the adaptive
// step choice is not differentiated).
//
//  k_adj_record    forward pass in the reference's loop shape (one thread per
//                  particle); every K segments the full particle state is
//                  written to a checkpoint pool (bump allocated, each
//                  checkpoint linked to the particle's previous one).
//  k_adj_backward  per particle, checkpoint blocks last to first: replay the
//                  block forward storing each segment's field polynomial and
//                  each accepted step (y, x, h); then walk the steps backward:
//                  recompute the 12 stages, propagate the adjoint through them
//                  and accumulate the moments sum(z), sum(z tau), sum(z tau^2)
//                  of z = dL/dOmega over the stages of the segment.  At the
//                  segment's start the moments are contracted with the
//                  segment's p0, v0 into dL/dG, dL/dB0, dL/dE (Omega is linear
//                  in them along the parabola), and per stage into dL/da,
//                  dL/dw when requested.
#include <cuda_runtime.h>
#include <stdint.h>

#include "st_device.cuh"

namespace st {


struct Ckpt {
  double t, px, py, pz, vx, vy, vz, Sx, Sy, Sz, h, next_gas, tempH, spare, tf;
  uint64_t rx, ry, rz, rw, n_coll, n_bounce, n_steps;
  int64_t seg, prev;
  int32_t fail, w, flags, pad;  // flags: has_spare | stop << 1 | fin << 2 | coll << 8 | wall << 16
};

// ---------------------------------------------------------------- walker
struct Walker {
  PState p;
  double tempH, tf;
  int w, wlast;
  bool fin;  // the previous segment ended its window
};

__device__ __forceinline__ void ckpt_write(Ckpt& c, const Walker& W, int64_t seg, int64_t prev) {
  c.t = W.p.t; c.px = W.p.px; c.py = W.p.py; c.pz = W.p.pz;
  c.vx = W.p.vx; c.vy = W.p.vy; c.vz = W.p.vz;
  c.Sx = W.p.Sx; c.Sy = W.p.Sy; c.Sz = W.p.Sz;
  c.h = W.p.h; c.next_gas = W.p.next_gas; c.tempH = W.tempH; c.spare = W.p.rng.spare; c.tf = W.tf;
  c.rx = W.p.rng.x; c.ry = W.p.rng.y; c.rz = W.p.rng.z; c.rw = W.p.rng.w;
  c.n_coll = W.p.n_coll; c.n_bounce = W.p.n_bounce; c.n_steps = W.p.n_steps;
  c.seg = seg; c.prev = prev;
  c.fail = W.p.fail; c.w = W.w;
  c.flags = (W.p.rng.has ? 1 : 0) | (W.p.stop ? 2 : 0) | (W.fin ? 4 : 0) | ((int)(uint8_t)W.p.coll << 8) |
            ((int)(uint8_t)W.p.wall << 16);
  c.pad = 0;
}

__device__ __forceinline__ void ckpt_read(const Ckpt& c, Walker& W, int wlast) {
  W.p.t = c.t; W.p.px = c.px; W.p.py = c.py; W.p.pz = c.pz;
  W.p.vx = c.vx; W.p.vy = c.vy; W.p.vz = c.vz;
  W.p.Sx = c.Sx; W.p.Sy = c.Sy; W.p.Sz = c.Sz;
  W.p.h = c.h; W.p.next_gas = c.next_gas; W.tempH = c.tempH; W.p.rng.spare = c.spare; W.tf = c.tf;
  W.p.rng.x = c.rx; W.p.rng.y = c.ry; W.p.rng.z = c.rz; W.p.rng.w = c.rw;
  W.p.n_coll = c.n_coll; W.p.n_bounce = c.n_bounce; W.p.n_steps = c.n_steps;
  W.p.fail = c.fail; W.w = c.w;
  W.p.rng.has = (c.flags & 1) != 0;
  W.p.stop = (c.flags & 2) != 0;
  W.fin = (c.flags & 4) != 0;
  W.p.coll = (char)((c.flags >> 8) & 0xff);
  W.p.wall = (char)((c.flags >> 16) & 0xff);
  W.wlast = wlast;
}

// Segment descriptor handed to the observer of the walk.
struct SegDesc {
  double t0, t1, o0[3], o1[3], p0[3], v0[3], y0[3], tempH0;
};

// One segment of the reference's window loop (src/particle.cpp:564-614) with
// an observer for every accepted DOP853 step.  Returns false when the particle
// has no segment left (all windows done, or stopped).
template <class OnSeg, class OnStep>
__device__ __forceinline__ bool walk_segment(Walker& W, const SetParams& P, OnSeg on_seg, OnStep on_step) {
  if (W.p.stop) return false;
  if (W.fin) {
    ++W.w;
    if (W.w >= W.wlast) return false;
    W.tf = ((double)W.w + 1.0) * P.ioutInt;
    W.tempH = W.p.h;
    W.fin = false;
  }
  SegStart s0;
  const bool fin = traj_event(W.p, P, W.tf, s0);
  if (W.p.fail == 0) {
    Seg g;
    seg_setup(g, P, s0, W.p.t);
    SegDesc d;
    d.t0 = s0.t; d.t1 = W.p.t;
    d.o0[0] = g.o0x; d.o0[1] = g.o0y; d.o0[2] = g.o0z;
    d.o1[0] = g.o1x; d.o1[1] = g.o1y; d.o1[2] = g.o1z;
    d.p0[0] = s0.px; d.p0[1] = s0.py; d.p0[2] = s0.pz;
    d.v0[0] = s0.vx; d.v0[1] = s0.vy; d.v0[2] = s0.vz;
    d.y0[0] = W.p.Sx; d.y0[1] = W.p.Sy; d.y0[2] = W.p.Sz;
    d.tempH0 = W.tempH;
    on_seg(d);
    dop_begin(g, P, W.p.Sx, W.p.Sy, W.p.Sz, W.tempH);
    int r;
    do {
      const double yx = W.p.Sx, yy = W.p.Sy, yz = W.p.Sz, x = g.x;
      r = dop_attempt(g, P, W.p.Sx, W.p.Sy, W.p.Sz);
      if (g.acc) on_step(yx, yy, yz, x, g.hu);
    } while (r == 0);
    W.tempH = g.h;
    if (P.keep) W.p.h = W.tempH;
    if (r < 0) {
      W.p.stop = true;
      W.p.fail = r;
    }
  }
  if (W.p.stop) {
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    W.p.t = nan;
    W.p.px = W.p.py = W.p.pz = nan;
    W.p.vx = W.p.vy = W.p.vz = nan;
    W.p.Sx = W.p.Sy = W.p.Sz = nan;
  }
  W.p.n_steps += 1;
  W.fin = fin;
  return true;
}

// ---------------------------------------------------------------- record
__global__ void k_adj_record(RunArgs a, AdjArgs b) {
  const int64_t nl = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.s.n; i += nl) {
    const SetParams& P = a.sets[a.s.set[i]];
    Walker W;
    W.p = load_state(a.s, i);
    W.w = 0;
    W.wlast = min(a.w_end, P.nwin);
    W.tf = 1.0 * P.ioutInt;
    W.tempH = W.p.h;
    W.fin = false;
    int64_t seg = 0, last = -1;
    if (W.wlast > 0) {
      while (true) {
        if (seg % b.k == 0) {
          const unsigned long long c = atomicAdd(b.pool_head, 1ull);
          if (c >= (unsigned long long)b.pool_cap) {
            atomicExch(b.overflow, 1);
            break;
          }
          ckpt_write(b.pool[c], W, seg, last);
          last = (int64_t)c;
        }
        if (!walk_segment(W, P, [](const SegDesc&) {}, [](double, double, double, double, double) {})) break;
        ++seg;
      }
    }
    b.last_ckpt[i] = last;
    b.nseg[i] = seg;
    store_state(a.s, i, W.p);
    a.s.w_done[i] = max(W.wlast, 0);
  }
}

// ---------------------------------------------------------------- adjoint step
namespace adj {
// stage inputs: for stage s (2..12) the earlier stages it sums and their
// coefficients; compile-time tables so every index resolves to a register
constexpr __device__ int kLst[13][9] = {
    {0}, {0}, {1}, {1, 2}, {1, 3}, {1, 3, 4}, {1, 4, 5}, {1, 4, 5, 6}, {1, 4, 5, 6, 7}, {1, 4, 5, 6, 7, 8},
    {1, 4, 5, 6, 7, 8, 9}, {1, 4, 5, 6, 7, 8, 9, 10}, {1, 4, 5, 6, 7, 8, 9, 10, 11}};
constexpr __device__ int kCnt[13] = {0, 0, 1, 2, 2, 3, 3, 4, 5, 6, 7, 8, 9};
constexpr __device__ double kA[13][9] = {
    {0}, {0}, {dop::A21}, {dop::A31, dop::A32}, {dop::A41, dop::A43}, {dop::A51, dop::A53, dop::A54},
    {dop::A61, dop::A64, dop::A65}, {dop::A71, dop::A74, dop::A75, dop::A76},
    {dop::A81, dop::A84, dop::A85, dop::A86, dop::A87},
    {dop::A91, dop::A94, dop::A95, dop::A96, dop::A97, dop::A98},
    {dop::A101, dop::A104, dop::A105, dop::A106, dop::A107, dop::A108, dop::A109},
    {dop::A111, dop::A114, dop::A115, dop::A116, dop::A117, dop::A118, dop::A119, dop::A1110},
    {dop::A121, dop::A124, dop::A125, dop::A126, dop::A127, dop::A128, dop::A129, dop::A1210, dop::A1211}};
// node of stage s (stage 12 at x + h)
constexpr __device__ double kC[13] = {0, 0, dop::C2, dop::C3, dop::C4, dop::C5, dop::C6, dop::C7, dop::C8,
                                      dop::C9, dop::C10, dop::C11, 1.0};
// 8th-order weights per stage
constexpr __device__ double kB[13] = {0, dop::B1, 0, 0, 0, 0, dop::B6, dop::B7, dop::B8, dop::B9, dop::B10,
                                      dop::B11, dop::B12};
}  // namespace adj

struct Moments {
  double z0[3], z1[3], z2[3];
  double ga, gw;
};

__device__ __forceinline__ void cross3(const double a[3], const double b[3], double r[3]) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}

__device__ __forceinline__ double stage_tau(int s, double tx, double h) {
  return (s == 1) ? tx : (s == 12 ? tx + h : fma(adj::kC[s], h, tx));
}

// Backward through one accepted DOP853 step from (x, y) with step h:
// lam (adjoint of the step's result) becomes the adjoint of y; the stages'
// dL/dOmega are accumulated into the segment moments.  The 12 stage states go
// to shared memory (ysm[(s * 3 + c) * BLOCK]), the stage derivatives and their
// adjoints stay in registers.
template <int BLOCK>
__device__ __forceinline__ void dop_step_adjoint(const Seg& g, const SetParams& P, double x, double h, const double y[3],
                                                 double lam[3], Moments& M, bool pulse, double* sm) {
  // sm[((s - 1) * 3 + c) * BLOCK]: stage state yy_s; sm[(36 + (s - 1) * 3 + c) * BLOCK]: k_s
#define ST_YS(s, c) sm[(((s)-1) * 3 + (c)) * BLOCK]
#define ST_KS(s, c) sm[(36 + ((s)-1) * 3 + (c)) * BLOCK]
  const double tx = x - g.t0;
  // forward recompute of the stages
#pragma unroll
  for (int s = 1; s <= 12; ++s) {
    double Y[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double acc = 0.0;
#pragma unroll
      for (int j = 0; j < adj::kCnt[s]; ++j) acc = fma(adj::kA[s][j], ST_KS(adj::kLst[s][j], c), acc);
      Y[c] = (s == 1) ? y[c] : fma(h, acc, y[c]);
      ST_YS(s, c) = Y[c];
    }
    double O[3], k[3];
    omega_at(g, P, stage_tau(s, tx, h), O[0], O[1], O[2]);
    bloch(Y[0], Y[1], Y[2], O[0], O[1], O[2], k[0], k[1], k[2]);
    ST_KS(s, 0) = k[0];
    ST_KS(s, 1) = k[1];
    ST_KS(s, 2) = k[2];
  }
  // backward: Kb[s] = dL/dk_s, pushed from the later stages
  double Kb[13][3];
#pragma unroll
  for (int s = 1; s <= 12; ++s)
#pragma unroll
    for (int c = 0; c < 3; ++c) Kb[s][c] = h * adj::kB[s] * lam[c];
#pragma unroll
  for (int s = 12; s >= 1; --s) {
    const double tau = stage_tau(s, tx, h);
    double O[3];
    omega_at(g, P, tau, O[0], O[1], O[2]);
    const double Y[3] = {ST_YS(s, 0), ST_YS(s, 1), ST_YS(s, 2)};
    double yb[3], z[3];
    cross3(O, Kb[s], yb);  // dL/dyy_s = Omega x kbar
    cross3(Kb[s], Y, z);   // dL/dOmega_s = kbar x yy
    const double tau2 = tau * tau;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      M.z0[c] += z[c];
      M.z1[c] = fma(z[c], tau, M.z1[c]);
      M.z2[c] = fma(z[c], tau2, M.z2[c]);
      lam[c] += yb[c];
    }
    if (pulse) {
      const double t = g.t0 + tau;
      double sn, cs;
      sincos(P.w * t, &sn, &cs);
      M.ga = fma(P.gamma * cs, z[2], M.ga);
      M.gw = fma(-P.gamma * P.a * t * sn, z[2], M.gw);
    }
#pragma unroll
    for (int j = 0; j < adj::kCnt[s]; ++j) {
      const int l = adj::kLst[s][j];
      const double ha = h * adj::kA[s][j];
#pragma unroll
      for (int c = 0; c < 3; ++c) Kb[l][c] = fma(ha, yb[c], Kb[l][c]);
    }
  }
#undef ST_YS
#undef ST_KS
}

// Contract a segment's moments into dL/dtheta (theta order of the file header);
// gth is strided by `stride` (shared memory, one column per thread).
__device__ __forceinline__ void contract(const SetParams& P, const double p0[3], const double v0[3], const Moments& M,
                                         double* gth, int stride) {
  const double gm = P.gamma;
  const double g_ = P.gravity ? kGravity : 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
#pragma unroll
    for (int j = 0; j < 3; ++j)
      gth[(3 * i + j) * stride] += gm * (M.z0[i] * p0[j] + M.z1[i] * v0[j] + (j == 1 ? 0.5 * g_ * M.z2[i] : 0.0));
    gth[(9 + i) * stride] += gm * M.z0[i];
  }
  // E: sum_s z_s x v_s with v_s = v0 + g tau_s yhat
  double zv[3];
  cross3(M.z0, v0, zv);
  const double ci = gm * P.inv_c2;
  gth[12 * stride] += ci * (zv[0] - g_ * M.z1[2]);
  gth[13 * stride] += ci * zv[1];
  gth[14 * stride] += ci * (zv[2] + g_ * M.z1[0]);
  gth[15 * stride] += M.ga;
  gth[16 * stride] += M.gw;
}

// ---------------------------------------------------------------- backward
constexpr int kSegF = kAdjSegF;  // t0 t1 o0[3] o1[3] p0[3] v0[3] y0[3] tempH0 step_start nsteps(-1: not stored, -2: none)

constexpr int kAdjBlock = 64;

__global__ void __launch_bounds__(kAdjBlock) k_adj_backward(RunArgs a, AdjArgs b) {
  __shared__ double ysm_all[2 * 12 * 3 * kAdjBlock];  // stage states, then stage derivatives
  __shared__ double gsm_all[kNumTheta * kAdjBlock];
  double* ysm = ysm_all + threadIdx.x;
  double* gth = gsm_all + threadIdx.x;  // gradient accumulators, stride kAdjBlock
  const int64_t nl = (int64_t)gridDim.x * blockDim.x;
  const int64_t lane = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double* sb = b.segbuf + lane * (int64_t)b.k * kSegF;
  double* st = b.stepbuf + lane * (int64_t)b.step_cap * 5;
  for (int64_t i = lane; i < a.s.n; i += nl) {
    const SetParams& P = a.sets[a.s.set[i]];
#pragma unroll
    for (int q = 0; q < kNumTheta; ++q) gth[q * kAdjBlock] = 0.0;
    double lam[3] = {b.dLdS[3 * i], b.dLdS[3 * i + 1], b.dLdS[3 * i + 2]};
    const bool live = a.s.stop[i] == 0 && (lam[0] != 0.0 || lam[1] != 0.0 || lam[2] != 0.0);
    int64_t ck = live ? b.last_ckpt[i] : -1;
    int64_t seg_end = b.nseg[i];
    const int wlast = min(a.w_end, P.nwin);
    while (ck >= 0) {
      if (ck >= b.pool_cap) {  // corrupt link: record and stop this particle
        atomicExch(b.overflow, 1);
        break;
      }
      const Ckpt C = b.pool[ck];
      const int64_t nblk64 = seg_end - C.seg;
      if (nblk64 < 0 || nblk64 > b.k) {  // block larger than the per-lane scratch
        atomicExch(b.overflow, 1);
        break;
      }
      const int nblk = (int)nblk64;
      // -- replay the block: segment descriptors, and the steps while they fit
      Walker W;
      ckpt_read(C, W, wlast);
      // the first half of the step buffer holds the block's steps; the second
      // half is the work area of segments replayed on their own
      const int half = b.step_cap / 2;
      int nstored = 0, jseg = -1;
      bool fits = true;
      for (int j = 0; j < nblk; ++j) {
        jseg = j;
        double* d = sb + (int64_t)j * kSegF;
        d[18] = (double)nstored;
        d[19] = -2.0;  // no descriptor (trajectory-only segment, e.g. sanity failure)
        const bool more = walk_segment(
            W, P,
            [&](const SegDesc& s) {
              d[0] = s.t0; d[1] = s.t1;
              d[2] = s.o0[0]; d[3] = s.o0[1]; d[4] = s.o0[2];
              d[5] = s.o1[0]; d[6] = s.o1[1]; d[7] = s.o1[2];
              d[8] = s.p0[0]; d[9] = s.p0[1]; d[10] = s.p0[2];
              d[11] = s.v0[0]; d[12] = s.v0[1]; d[13] = s.v0[2];
              d[14] = s.y0[0]; d[15] = s.y0[1]; d[16] = s.y0[2];
              d[17] = s.tempH0;
              d[19] = fits ? 0.0 : -1.0;
            },
            [&](double yx, double yy, double yz, double x, double h) {
              if (fits && nstored < half) {
                double* e = st + (int64_t)nstored * 5;
                e[0] = yx; e[1] = yy; e[2] = yz; e[3] = x; e[4] = h;
                ++nstored;
                d[19] += 1.0;
              } else {
                fits = false;
                d[19] = -1.0;
              }
            });
        if (!more) {
          d[19] = -2.0;
          break;
        }
      }
      (void)jseg;
      // -- backward over the block's segments
      for (int j = nblk - 1; j >= 0; --j) {
        const double* d = sb + (int64_t)j * kSegF;
        if (d[19] == -2.0) continue;
        Seg g;
        const double o0[3] = {d[2], d[3], d[4]};
        const double o1[3] = {d[5], d[6], d[7]};
        seg_begin(g, P, d[0], d[1], o0, o1);
        Moments M;
#pragma unroll
        for (int c = 0; c < 3; ++c) M.z0[c] = M.z1[c] = M.z2[c] = 0.0;
        M.ga = M.gw = 0.0;
        if (d[19] >= 0.0) {
          const int s0 = (int)d[18], ns = (int)d[19];
          for (int k = ns - 1; k >= 0; --k) {
            const double* e = st + (int64_t)(s0 + k) * 5;
            const double y[3] = {e[0], e[1], e[2]};
            dop_step_adjoint<kAdjBlock>(g, P, e[3], e[4], y, lam, M, b.pulse_grads != 0, ysm);
          }
        } else {
          // steps did not fit: replay this segment alone, in chunks of step_cap
          // accepted steps, last chunk first
          int total = 0;
          {
            Seg r = g;
            double S[3] = {d[14], d[15], d[16]};
            dop_begin(r, P, S[0], S[1], S[2], d[17]);
            int rc;
            do {
              rc = dop_attempt(r, P, S[0], S[1], S[2]);
              if (r.acc) ++total;
            } while (rc == 0);
          }
          double* wk = st + (int64_t)half * 5;
          for (int hi = total; hi > 0; hi -= half) {
            const int lo = max(0, hi - half);
            Seg r = g;
            double S[3] = {d[14], d[15], d[16]};
            dop_begin(r, P, S[0], S[1], S[2], d[17]);
            int idx = 0, rc;
            do {
              const double yx = S[0], yy = S[1], yz = S[2], x = r.x;
              rc = dop_attempt(r, P, S[0], S[1], S[2]);
              if (r.acc) {
                if (idx >= lo && idx < hi) {
                  double* e = wk + (int64_t)(idx - lo) * 5;
                  e[0] = yx; e[1] = yy; e[2] = yz; e[3] = x; e[4] = r.hu;
                }
                ++idx;
              }
            } while (rc == 0 && idx < hi);
            for (int k = hi - lo - 1; k >= 0; --k) {
              const double* e = wk + (int64_t)k * 5;
              const double y[3] = {e[0], e[1], e[2]};
              dop_step_adjoint<kAdjBlock>(g, P, e[3], e[4], y, lam, M, b.pulse_grads != 0, ysm);
            }
          }
        }
        const double p0[3] = {d[8], d[9], d[10]};
        const double v0[3] = {d[11], d[12], d[13]};
        contract(P, p0, v0, M, gth, kAdjBlock);
      }
      seg_end = C.seg;
      ck = C.prev;
    }
#pragma unroll
    for (int q = 0; q < kNumTheta; ++q) b.grad[i * kNumTheta + q] = gth[q * kAdjBlock];
  }
}

// ---------------------------------------------------------------- launchers
int launch_adj_record(const RunArgs& a, const AdjArgs& b, int blocks, void* stream) {
  if (a.s.n == 0) return 0;
  k_adj_record<<<blocks, 128, 0, (cudaStream_t)stream>>>(a, b);
  return (int)cudaGetLastError();
}

int launch_adj_backward(const RunArgs& a, const AdjArgs& b, int blocks, void* stream) {
  if (a.s.n == 0) return 0;
  k_adj_backward<<<blocks, kAdjBlock, 0, (cudaStream_t)stream>>>(a, b);
  return (int)cudaGetLastError();
}

size_t adj_ckpt_bytes() { return sizeof(Ckpt); }

}  // namespace st
