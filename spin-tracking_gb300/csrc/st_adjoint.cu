// Discrete adjoint of the DOP853 (and Magnus CFET8) spin integration along the
// particles' fixed trajectories: gradients of a loss L(S_final) with respect
// to the field parameters theta = [Gx(3), Gy(3), Gz(3), B0(3), E(3), a, w].
//
// The trajectory does not depend on theta, and with the accepted step
// sequence held fixed every DOP853 step is a linear map of the spin, so the
// gradient is the exact derivative of the discrete forward map (the adaptive
// step choice is not differentiated).
//
// The forward pass (the trajectory-ahead kernel with its tape switch on, see
// st_kernels.cu) writes every particle's accepted steps (y, x, h) and
// integrated segments (t0, p0, v0) to a paged tape in device memory.
// k_adj_backward walks each particle's tape last step first, one step adjoint
// per loop iteration on every lane (lanes converge: every iteration is the
// same arithmetic).  A step adjoint recomputes the 12 stages, propagates the
// adjoint through them and accumulates the moments sum(z), sum(z tau),
// sum(z tau^2) of z = dL/dOmega over the segment's stages.  At the segment's
// first step the moments are contracted with the segment's p0, v0 into dL/dG,
// dL/dB0, dL/dE (Omega is linear in them along the parabola), and per stage
// into dL/da, dL/dw when requested.
#include <cuda_runtime.h>
#include <stdint.h>

#include "st_device.cuh"

namespace st {

// ---------------------------------------------------------------- adjoint step
// The stage structure (dopst::src, cnt, a, c, b) is shared with the forward stepper (st_device.cuh).

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
  return (s == 1) ? tx : (s == 12 ? tx + h : fma(dopst::c(s), h, tx));
}

// Backward through one accepted DOP853 step from (x, y) with step h:
// lam (the adjoint of the step's result) becomes the adjoint of y, and the
// stages' dL/dOmega are accumulated into the segment moments.  The stages are
// recomputed as the forward step computed them; their derivatives stay in
// registers, their states and fields go to shared memory (sm[(s * 3 + c) *
// BLOCK]) for the backward sweep.  With kh_s = (dL/dk_s) / h:
//   kh_s = b_s lam + sum_{r > s} a_rs yb_r,  yb_s = Omega_s x (h kh_s),
//   z_s = (h kh_s) x Y_s,  dL/dy = lam + sum_s yb_s.
template <int BLOCK>
__device__ __forceinline__ void dop_step_adjoint(const Seg& g, const SetParams& P, double x, double h, const double y[3],
                                                 double lam[3], Moments& M, bool pulse, double* sm) {
#define ST_YS(s, c) sm[(((s)-1) * 3 + (c)) * BLOCK]
#define ST_OS(s, c) sm[(36 + ((s)-1) * 3 + (c)) * BLOCK]
  const double tx = x - g.t0;
  // ---- forward: the 12 stages
  double K[11][3];  // k_1 .. k_11
#pragma unroll
  for (int s = 1; s <= 12; ++s) {
    double Y[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      if (s == 1) {
        Y[c] = y[c];
      } else {
        double acc = dopst::a(s, 0) * K[dopst::src(s, 0) - 1][c];
#pragma unroll
        for (int j = 1; j < dopst::cnt(s); ++j) acc = fma(dopst::a(s, j), K[dopst::src(s, j) - 1][c], acc);
        Y[c] = fma(h, acc, y[c]);
      }
      ST_YS(s, c) = Y[c];
    }
    double O[3];
    omega_at(g, P, stage_tau(s, tx, h), O[0], O[1], O[2]);
    ST_OS(s, 0) = O[0];
    ST_OS(s, 1) = O[1];
    ST_OS(s, 2) = O[2];
    if (s < 12) bloch(Y[0], Y[1], Y[2], O[0], O[1], O[2], K[s - 1][0], K[s - 1][1], K[s - 1][2]);
  }
  // ---- backward sweep, stage 12 first
  double kh[12][3];
#pragma unroll
  for (int s = 1; s <= 12; ++s)
#pragma unroll
    for (int c = 0; c < 3; ++c) kh[s - 1][c] = (dopst::b(s) != 0.0) ? dopst::b(s) * lam[c] : 0.0;
#pragma unroll
  for (int s = 12; s >= 1; --s) {
    const double kb[3] = {h * kh[s - 1][0], h * kh[s - 1][1], h * kh[s - 1][2]};
    const double O[3] = {ST_OS(s, 0), ST_OS(s, 1), ST_OS(s, 2)};
    const double Y[3] = {ST_YS(s, 0), ST_YS(s, 1), ST_YS(s, 2)};
    double yb[3], z[3];
    cross3(O, kb, yb);  // dL/dY_s
    cross3(kb, Y, z);   // dL/dOmega_s
    const double tau = stage_tau(s, tx, h);
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
    for (int j = 0; j < dopst::cnt(s); ++j) {
      const int l = dopst::src(s, j) - 1;
#pragma unroll
      for (int c = 0; c < 3; ++c) kh[l][c] = fma(dopst::a(s, j), yb[c], kh[l][c]);
    }
  }
#undef ST_YS
#undef ST_OS
}

// Rodrigues rotation v' = R(k) v = v cos a + (v x k) sin(a)/a + k (k.v)(1 - cos a)/a^2
// (a = |k|, rodrigues in st_device.cuh): given mu = dL/dv', return dL/dk in gk
// and replace mu by dL/dv = R(k)^T mu = R(-k) mu.  With al = cos a,
// be = sin(a)/a, ga = (1 - cos a)/a^2 and their a-derivatives,
//   dL/dk = k/a (al' v.mu + be' (v x k).mu + ga' (k.v)(k.mu)) + be (mu x v)
//           + ga ((k.mu) v + (k.v) mu).
__device__ __forceinline__ void rodrigues_adjoint(const double k[3], const double v[3], double mu[3], double gk[3]) {
  const double a2 = fma(k[2], k[2], fma(k[1], k[1], k[0] * k[0]));
  const double r = rsqrt(a2);
  const double a = a2 * r;
  double s, c;
  sincos(a, &s, &c);
  const double omc = 1.0 - c;
  const double be = s * r, ga = omc * (r * r);
  const double dal = -s;
  const double dbe = (a * c - s) * (r * r);
  const double dga = (a * s - 2.0 * omc) * (r * r * r);
  const double vm = v[0] * mu[0] + v[1] * mu[1] + v[2] * mu[2];
  const double kv = k[0] * v[0] + k[1] * v[1] + k[2] * v[2];
  const double km = k[0] * mu[0] + k[1] * mu[1] + k[2] * mu[2];
  double vk[3], mv[3], mk[3];
  cross3(v, k, vk);
  cross3(mu, v, mv);
  cross3(mu, k, mk);
  const double vkm = vk[0] * mu[0] + vk[1] * mu[1] + vk[2] * mu[2];
  const double coef = (dal * vm + dbe * vkm + dga * kv * km) * r;
#pragma unroll
  for (int q = 0; q < 3; ++q) gk[q] = fma(coef, k[q], fma(be, mv[q], ga * fma(km, v[q], kv * mu[q])));
  // R(-k) mu = mu cos a - (mu x k) sin(a)/a + k (k.mu)(1 - cos a)/a^2
  const double d = km * ga;
#pragma unroll
  for (int q = 0; q < 3; ++q) mu[q] = fma(k[q], d, fma(-be, mk[q], mu[q] * c));
}

// Backward through one accepted Magnus CFET8 step from (x, y) with step h
// (magnus_stages in st_device.cuh; the CFET6 companion only estimated the
// error and does not enter the accepted map): the field at the five
// Gauss-Legendre nodes is recomputed, the 11 rotations are replayed with
// their inputs kept in shared memory (sm[(n * 3 + c) * BLOCK]), then undone
// last first, each giving dL/dk_n; dL/d(h Omega_j) = sum_n G_nj dL/dk_n and
// z_j = h dL/d(h Omega_j) is dL/dOmega at node j, accumulated into the
// segment moments like the DOP853 stages.
template <int BLOCK>
__device__ __forceinline__ void magnus_step_adjoint(const Seg& g, const SetParams& P, double x, double h,
                                                    const double y[3], double lam[3], Moments& M, bool pulse,
                                                    double* sm) {
#define ST_VN(n, c) sm[((n) * 3 + (c)) * BLOCK]
  const double tx = x - g.t0;
  double B[5][3];
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    omega_at(g, P, fma(cfetc::x(i), h, tx), B[i][0], B[i][1], B[i][2]);
#pragma unroll
    for (int c = 0; c < 3; ++c) B[i][c] *= h;
  }
  double v[3] = {y[0], y[1], y[2]};
#pragma unroll 1
  for (int n = 0; n < 11; ++n) {
    const double* cf = kMagnusExp[n];
    double k[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double s = cf[0] * B[0][c];
#pragma unroll
      for (int j = 1; j < 5; ++j) s = fma(cf[j], B[j][c], s);
      k[c] = s;
      ST_VN(n, c) = v[c];
    }
    rodrigues(k[0], k[1], k[2], v[0], v[1], v[2]);
  }
  double zb[5][3] = {};  // dL/d(h Omega_j)
#pragma unroll 1
  for (int n = 10; n >= 0; --n) {
    const double* cf = kMagnusExp[n];
    double k[3], vn[3], gk[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      double s = cf[0] * B[0][c];
#pragma unroll
      for (int j = 1; j < 5; ++j) s = fma(cf[j], B[j][c], s);
      k[c] = s;
      vn[c] = ST_VN(n, c);
    }
    rodrigues_adjoint(k, vn, lam, gk);
#pragma unroll
    for (int j = 0; j < 5; ++j)
#pragma unroll
      for (int c = 0; c < 3; ++c) zb[j][c] = fma(cf[j], gk[c], zb[j][c]);
  }
#pragma unroll
  for (int j = 0; j < 5; ++j) {
    const double tau = fma(cfetc::x(j), h, tx);
    const double tau2 = tau * tau;
    double z[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      z[c] = h * zb[j][c];
      M.z0[c] += z[c];
      M.z1[c] = fma(z[c], tau, M.z1[c]);
      M.z2[c] = fma(z[c], tau2, M.z2[c]);
    }
    if (pulse) {
      const double t = g.t0 + tau;
      double sn, cs;
      sincos(P.w * t, &sn, &cs);
      M.ga = fma(P.gamma * cs, z[2], M.ga);
      M.gw = fma(-P.gamma * P.a * t * sn, z[2], M.gw);
    }
  }
#undef ST_VN
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
constexpr int kAdjBlock = 64;

// Record the first tape inconsistency (later ones are dropped).
__device__ void tape_report(const TapeArgs& t, int code, int64_t i, int sp, int si, int gp, int gi, long long ws,
                            long long wg) {
  if (atomicCAS(reinterpret_cast<unsigned long long*>(t.error), 0ull, (unsigned long long)code) != 0ull) return;
  t.error[1] = i;
  t.error[2] = sp;
  t.error[3] = si;
  t.error[4] = gp;
  t.error[5] = gi;
  t.error[6] = t.nsteps[i];
  t.error[7] = t.nsegs[i];
  t.error[8] = ws;
  t.error[9] = wg;
}

// Field polynomial of tape segment record (page, idx).
__device__ __forceinline__ void tape_load_seg(const TapeArgs& t, const SetParams& P, int page, int idx, Seg& g) {
  const double* r = t.pool + (size_t)page * kTapePageD + (size_t)idx * kTapeSegD;
  double o0[3], o1[3];
  seg_field(P, r[1], r[2], r[3], r[4], r[5], r[6], o0, o1);
  seg_begin(g, P, r[0], r[0], o0, o1);
}

// Lane state machine: fetch a particle from the work order (divergent, once
// per particle), then one step adjoint per iteration until its tape is
// exhausted.  Reads lam and grad at the fetch and writes both back when the
// particle's piece of tape is done, so a backward in pieces (replayed
// intervals, a kept tail) continues each gradient sum in the order of a
// backward over the whole tape, bit for bit; the tape's consistency (both chains end together, page indices inside the pool) is
// checked and a violation sets t.error and abandons the particle.
// MAGNUS: the tape holds Magnus CFET8 steps (integratorType 2) instead of DOP853 ones.
template <bool MAGNUS>
__global__ void __launch_bounds__(kAdjBlock) k_adj_backward(RunArgs a, TapeArgs t) {
  __shared__ double stage_all[2 * 12 * 3 * kAdjBlock];  // stage states, then stage fields
  __shared__ double gsm_all[kNumTheta * kAdjBlock];
  double* stg = stage_all + threadIdx.x;
  double* gth = gsm_all + threadIdx.x;  // gradient accumulators, stride kAdjBlock
  const unsigned FULL = 0xffffffffu;
  const bool pulse = t.pulse_grads != 0;
  const int64_t pages = t.pool_pages;
  bool active = false, done = false;
  int64_t i = 0;
  const SetParams* P = a.sets;
  Seg g;
  Moments M;
  double lam[3] = {0.0, 0.0, 0.0};
  int sp = -1, si = 0, gp = -1, gi = 0;
  long long walked_s = 0, walked_g = 0;  // records of the particle's tape walked so far
  while (true) {
    // ---- fetch
    while (!active && !done) {
      const unsigned long long item = atomicAdd(&a.status->queue_head, 1ull);
      if (item >= (unsigned long long)a.nitems) {
        done = true;
        break;
      }
      i = a.order ? a.order[item] : (int64_t)item;
      if (t.final_stop[i]) continue;  // stopped particles keep a zero gradient
      if (!t.complete[i]) {
        tape_report(t, 1, i, -1, -1, -1, -1, 0, 0);
        continue;
      }
      lam[0] = t.lam[3 * i];
      lam[1] = t.lam[3 * i + 1];
      lam[2] = t.lam[3 * i + 2];
      if (t.nsteps[i] == 0 || (lam[0] == 0.0 && lam[1] == 0.0 && lam[2] == 0.0)) continue;
      sp = t.step_page[i];
      si = t.step_fill[i] - 1;
      gp = t.seg_page[i];
      gi = t.seg_fill[i] - 1;
      if (sp < 0 || sp >= pages || gp < 0 || gp >= pages || si < 0 || gi < 0) {
        tape_report(t, 2, i, sp, si, gp, gi, 0, 0);
        continue;
      }
      P = &a.sets[a.s.set[i]];
      tape_load_seg(t, *P, gp, gi, g);
#pragma unroll
      for (int q = 0; q < kNumTheta; ++q) gth[q * kAdjBlock] = t.grad[i * kNumTheta + q];
#pragma unroll
      for (int c = 0; c < 3; ++c) M.z0[c] = M.z1[c] = M.z2[c] = 0.0;
      M.ga = M.gw = 0.0;
      walked_s = walked_g = 0;
      active = true;
    }
    if (__all_sync(FULL, done)) break;
    if (!active) continue;
    // ---- one step adjoint
    const double* r = t.pool + (size_t)sp * kTapePageD + (size_t)si * kTapeStepD;
    const double y[3] = {r[0], r[1], r[2]};
    const double x = r[3], h = r[4];
    const bool first = x == g.t0;  // the segment's first step starts at its t0
    if (MAGNUS)
      magnus_step_adjoint<kAdjBlock>(g, *P, x, h, y, lam, M, pulse, stg);
    else
      dop_step_adjoint<kAdjBlock>(g, *P, x, h, y, lam, M, pulse, stg);
    ++walked_s;
    bool finish = false;
    int bad = 0;
    if (--si < 0) {  // chains link to earlier allocated pages: indices strictly decrease
      const int nsp = t.page_prev[sp];
      if (nsp >= sp) bad = 5;
      sp = bad ? -1 : nsp;
      si = kTapeStepsPerPage - 1;
    }
    if (bad) {
      finish = true;
    } else if (first) {
      const double* sr = t.pool + (size_t)gp * kTapePageD + (size_t)gi * kTapeSegD;
      const double p0[3] = {sr[1], sr[2], sr[3]};
      const double v0[3] = {sr[4], sr[5], sr[6]};
      contract(*P, p0, v0, M, gth, kAdjBlock);
#pragma unroll
      for (int c = 0; c < 3; ++c) M.z0[c] = M.z1[c] = M.z2[c] = 0.0;
      M.ga = M.gw = 0.0;
      ++walked_g;
      if (--gi < 0) {
        const int ngp = t.page_prev[gp];
        if (ngp >= gp) bad = 5;
        gp = ngp;
        gi = kTapeSegsPerPage - 1;
      }
      if (bad) {
        finish = true;
      } else if (gp < 0) {
        finish = true;
        if (sp >= 0) bad = 3;  // steps left without a segment
      } else if (gp >= pages || sp >= pages) {
        finish = true;
        bad = 5;
      } else if (sp < 0) {
        finish = true;
        bad = 4;  // a segment left without steps
      } else {
        tape_load_seg(t, *P, gp, gi, g);
      }
    } else if (sp < 0 || sp >= pages) {
      finish = true;
      bad = sp < 0 ? 6 : 5;  // the segment's first step is missing
    }
    if (finish) {
      if (bad) tape_report(t, bad, i, sp, si, gp, gi, walked_s, walked_g);
      t.lam[3 * i] = lam[0];
      t.lam[3 * i + 1] = lam[1];
      t.lam[3 * i + 2] = lam[2];
#pragma unroll
      for (int q = 0; q < kNumTheta; ++q) t.grad[i * kNumTheta + q] = gth[q * kAdjBlock];
      active = false;
    }
  }
}

// ---------------------------------------------------------------- launchers
int adj_backward_block() { return kAdjBlock; }

int adj_backward_max_blocks_per_sm(int magnus) {
  int nb = 0;
  if (magnus)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_adj_backward<true>, kAdjBlock, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_adj_backward<false>, kAdjBlock, 0);
  return nb;
}

int launch_adj_backward(const RunArgs& a, const TapeArgs& t, int blocks, int magnus, void* stream) {
  if (a.nitems == 0) return 0;
  if (magnus)
    k_adj_backward<true><<<blocks, kAdjBlock, 0, (cudaStream_t)stream>>>(a, t);
  else
    k_adj_backward<false><<<blocks, kAdjBlock, 0, (cudaStream_t)stream>>>(a, t);
  return (int)cudaGetLastError();
}

}  // namespace st
