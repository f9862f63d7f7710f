// integratorType 6: the noise spectrum of the field each particle sees.
//
// The reference (src/particle.cpp:746-824, src/integrator.cpp:724-743,
// src/floquet.cpp:25-156) integrates no spin for this type.  Along every
// trajectory segment it samples the noise field
//   x(t) = gamma (v x E / c^2 + grad(p) + testNoise(t)) / 2
// on the grid of multiples of the particle's step h and feeds it to a
// per-particle aggregator of 17 Goertzel recursions, one per frequency of the
// dressed-spin Floquet analysis (floquet_diagonalize: the eigenphase of the
// one-period propagator of gamma (B0 + pulse) gives the splitting dE, and the
// frequencies are k w + {-dE, 0, dE}).  Per frequency and field component the
// aggregator keeps the recursion's last two values s1, s2 and the Laplace
// term of the covariance diagonal; it restarts at every window.
//
// Here one warp serves one particle: lane k < 17 owns frequency k and keeps
// its nine accumulators in registers for the whole window, while every lane
// runs the (identical) trajectory.  The noise field and the recursions use the
// reference's operations in its order without contraction, so a run without
// test noise matches the reference's aggregators bit for bit; with test noise
// the device's sin of w t enters.  What this file leaves to the caller: the
// reference's reduction of the per-particle covariances (its CPU loop nests
// the tree the wrong way round, src/particle.cpp:826-834, and its GPU path does
// not reduce) is replaced by a plain sum over particles (st_covariance_spectrum
// in st_api.cpp), and the Floquet master equation that turns the spectrum into
// b_end (src/integrator.cpp:790-890, Eigen's matrix exponential) is not built.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "st_device.cuh"
#include "st_engine.cuh"
#include "st_tableau.h"

namespace st {

// ---------------------------------------------------------------- host: Floquet frequencies
namespace {

struct HVec {
  double x, y, z;
};
struct HQuat {
  double w, x, y, z;
};
inline HVec hv(double x, double y, double z) { return {x, y, z}; }
inline HVec hadd(HVec a, HVec b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline HVec hscale(double s, HVec a) { return {a.x * s, a.y * s, a.z * s}; }
inline HVec hcross(HVec a, HVec b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline double hdot(HVec a, HVec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// qMult (src/quaternion.cpp)
inline HQuat hqmul(HQuat a, HQuat b) {
  return {a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
          a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z, a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x};
}
// rodriguezQuat (src/quaternion.cpp:150-156): rotation by |k| dt about -k/|k|
inline HQuat hrot(HVec k, double dt) {
  const double angle = sqrt(k.x * k.x + k.y * k.y + k.z * k.z);
  HVec n = {k.x / angle, k.y / angle, k.z / angle};
  const double h = angle * dt;
  n = hscale(-sin(h / 2.0), n);
  return {cos(h / 2.0), n.x, n.y, n.z};
}

// findCrossTerm (src/integrator.cpp:63-70) for a particle at rest at the
// origin at t0: the field of the dressed spin (interpolate, :48-61, moves it
// only under gravity).
HVec cross_term(const st_options& o, double t, double t0) {
  HVec p = hv(0.0, 0.0, 0.0), v = hv(0.0, 0.0, 0.0);
  if (o.gravity) {
    const HVec a = hv(0.0, kGravity, 0.0);
    p = hadd(hadd(p, hscale(t - t0, v)), hscale(t - t0, hscale(t - t0, hscale(0.5, a))));
    v = hadd(v, hscale(t - t0, a));
  }
  const HVec Gx = hv(o.Gx.x, o.Gx.y, o.Gx.z), Gy = hv(o.Gy.x, o.Gy.y, o.Gy.z), Gz = hv(o.Gz.x, o.Gz.y, o.Gz.z);
  const HVec G = hv(hdot(p, Gx), hdot(p, Gy), hdot(p, Gz));
  const HVec pulse = hv(0.0, 0.0, o.a * cos(o.w * t));
  const HVec E = hv(o.E.x, o.E.y, o.E.z), B0 = hv(o.B0.x, o.B0.y, o.B0.z);
  const HVec B = hadd(hadd(hadd(pulse, B0), hscale(1.0 / kC2, hcross(v, E))), G);
  return hscale(o.gamma, B);
}

// sum_j c_j B_j with the five coefficients taken forwards or backwards
HVec exponent(const double c[5], bool rev, const HVec B[5]) {
  HVec s = hscale(c[rev ? 4 : 0], B[0]);
  for (int j = 1; j < 5; ++j) s = hadd(s, hscale(c[rev ? 4 - j : j], B[j]));
  return s;
}

// integrateHamiltonian (src/integrator.cpp:745-785): y = q1 q2 ... q11 y per
// CFET8 step of h over [t0, tf].
int hamiltonian(const st_options& o, double t0, double tf, HQuat& y, double h) {
  using namespace cfet;
  static const double G[6][5] = {{G11, G12, G13, G14, G15}, {G21, G22, G23, G24, G25}, {G31, G32, G33, G34, G35},
                                 {G41, G42, G43, G44, G45}, {G51, G52, G53, G54, G55}, {G61, G62, G63, G64, G65}};
  static const double X[5] = {X1, X2, X3, X4, X5};
  double t = t0;
  unsigned int nstep = 0;
  while (t < tf) {
    nstep++;
    if (nstep > o.nmax) return -2;
    const double rest = tf - t;
    if (h >= rest) h = rest;
    HVec B[5];
    for (int i = 0; i < 5; ++i) B[i] = cross_term(o, t + X[i] * h, t0);
    HQuat q[12];
    for (int r = 0; r < 5; ++r) q[11 - r] = hrot(exponent(G[r], true, B), h);  // q11 .. q7
    for (int r = 5; r >= 0; --r) q[r + 1] = hrot(exponent(G[r], false, B), h);  // q6 .. q1
    HQuat prod = hqmul(q[1], q[2]);
    for (int r = 3; r <= 11; ++r) prod = hqmul(prod, q[r]);
    y = hqmul(prod, y);
    t += h;
  }
  return 0;
}

}  // namespace

int floquet_frequencies(const st_options& o, double freq[kSpecFreqs], double* dt) {
  if (!(o.w != 0.0) || !std::isfinite(o.w)) return -1;  // no period: the reference's loop would not end
  const double t0 = 0.0, tf = (2 * M_PI) / o.w;
  const int n_prop = 100;
  HQuat y = {1.0, 0.0, 0.0, 0.0};
  for (int i = 0; i < n_prop; ++i) {
    const double t1 = t0 + (tf - t0) * i / n_prop;
    const double t2 = t0 + (tf - t0) * (i + 1) / n_prop;
    hamiltonian(o, t1, t2, y, 1e-6);
  }
  // qEigenval (src/quaternion.cpp:169-172) of the period's propagator
  const double ez = -sqrt(1.0 - y.w * y.w);
  const double ea = fabs(atan2(ez, y.w)) / (tf - t0);
  const double eb = -ea;
  const double deltaE = ea - eb;
  for (int k = 0; k <= 11 / 2; ++k)
    for (int i = -1; i < 2; ++i) {
      const int index = k * 3 + i;
      if (index >= 0) freq[index] = deltaE * i + k * o.w;
    }
  *dt = (tf - t0) / n_prop;
  return 0;
}

int build_spec_set(const st_options& o, SpecSet* q) {
  double f[kSpecFreqs], dt = 0.0;
  if (floquet_frequencies(o, f, &dt) != 0) return -1;
  for (int k = 0; k < kSpecFreqs; ++k) {
    q->freq[k] = f[k];
    // goertzel_stage_1 / _2 (src/floquet.cpp:25-38) evaluate these per sample
    const double angle = f[k] * dt;
    q->two_cos[k] = 2 * cos(angle);
    q->sin_a[k] = sin(angle);
  }
  q->fdt = dt;
  q->na[0] = o.noiseAmplitudes.x; q->na[1] = o.noiseAmplitudes.y; q->na[2] = o.noiseAmplitudes.z;
  q->nw[0] = o.noiseFrequencies.x; q->nw[1] = o.noiseFrequencies.y; q->nw[2] = o.noiseFrequencies.z;
  return 0;
}

// ---------------------------------------------------------------- device
// The noise field at t of a segment starting at (t0, p0, v0), halved:
// findNoiseTerm (src/integrator.cpp:72-80) in the reference's operation order.
__device__ __forceinline__ void noise_sample(const SetParams& P, const SpecSet& Q, const SegStart& s0, double t,
                                             double& xx, double& xy, double& xz) {
  const double d = __dsub_rn(t, s0.t);
  double px = __dadd_rn(s0.px, __dmul_rn(d, s0.vx));
  double py = __dadd_rn(s0.py, __dmul_rn(d, s0.vy));
  double pz = __dadd_rn(s0.pz, __dmul_rn(d, s0.vz));
  double vx = s0.vx, vy = s0.vy, vz = s0.vz;
  if (P.gravity) {
    px = __dadd_rn(px, __dmul_rn(d, __dmul_rn(d, __dmul_rn(0.0, 0.5))));
    py = __dadd_rn(py, __dmul_rn(d, __dmul_rn(d, __dmul_rn(kGravity, 0.5))));
    pz = __dadd_rn(pz, __dmul_rn(d, __dmul_rn(d, __dmul_rn(0.0, 0.5))));
    vx = __dadd_rn(vx, __dmul_rn(d, 0.0));
    vy = __dadd_rn(vy, __dmul_rn(d, kGravity));
    vz = __dadd_rn(vz, __dmul_rn(d, 0.0));
  }
  auto dot3 = [](double ax, double ay, double az, const double* g) {
    return __dadd_rn(__dadd_rn(__dmul_rn(ax, g[0]), __dmul_rn(ay, g[1])), __dmul_rn(az, g[2]));
  };
  const double gx = dot3(px, py, pz, P.Gx), gy = dot3(px, py, pz, P.Gy), gz = dot3(px, py, pz, P.Gz);
  const double cx = __dsub_rn(__dmul_rn(vy, P.Ez), __dmul_rn(vz, P.Ey));
  const double cy = __dsub_rn(__dmul_rn(vz, P.Ex), __dmul_rn(vx, P.Ez));
  const double cz = __dsub_rn(__dmul_rn(vx, P.Ey), __dmul_rn(vy, P.Ex));
  const double nx = __dmul_rn(Q.na[0], sin(__dmul_rn(Q.nw[0], t)));
  const double ny = __dmul_rn(Q.na[1], sin(__dmul_rn(Q.nw[1], t)));
  const double nz = __dmul_rn(Q.na[2], sin(__dmul_rn(Q.nw[2], t)));
  const double bx = __dadd_rn(__dadd_rn(__dmul_rn(cx, P.inv_c2), gx), nx);
  const double by = __dadd_rn(__dadd_rn(__dmul_rn(cy, P.inv_c2), gy), ny);
  const double bz = __dadd_rn(__dadd_rn(__dmul_rn(cz, P.inv_c2), gz), nz);
  xx = __ddiv_rn(__dmul_rn(bx, P.gamma), 2.0);
  xy = __ddiv_rn(__dmul_rn(by, P.gamma), 2.0);
  xz = __ddiv_rn(__dmul_rn(bz, P.gamma), 2.0);
}

// One window (window >= 0) or up to next_t (window < 0) of every particle of
// a spectrum context: one warp per particle, lane k < kSpecFreqs owning
// Goertzel frequency k.  Trajectory, window bookkeeping and failure codes as
// the plain kernel (n_steps counts segments); S is not integrated.
template <bool GAS>
__global__ void __launch_bounds__(kSpecBlock) k_spectrum(RunArgs a, int window, double next_t, SpecArgs sp) {
  const int lane = threadIdx.x & 31;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  unsigned long long n_seg = 0;
  bool hit = false;
  const unsigned long long dl = run_deadline(a);
  if (i < a.s.n) {  // uniform over the warp
    const int set = a.s.set[i];
    const SetParams& P = a.sets[set];
    const SpecSet& Q = sp.sets[set];
    double tf = next_t;
    bool run = true;
    if (window >= 0) {
      run = window < P.nwin && a.s.w_done[i] == window;
      tf = ((double)window + 1.0) * P.ioutInt;
    }
    if (run) {
      const int k = lane < kSpecFreqs ? lane : 0;  // lanes past the frequencies shadow frequency 0
      const double c2 = Q.two_cos[k], sn = Q.sin_a[k];
      double s1x = 0.0, s1y = 0.0, s1z = 0.0, s2x = 0.0, s2y = 0.0, s2z = 0.0;
      double imx = 0.0, imy = 0.0, imz = 0.0;
      long long ns = 0;
      PState p = load_state(a.s, i);
      const double hs = p.h;  // the sampling step (integrateSpectrum's h)
      bool finished = false;
      unsigned int guard = 0;
      while (!finished && !p.stop && !hit) {
        SegStart s0;
        finished = traj_event<false, GAS>(p, P, tf, s0);
        ++n_seg;
        if (p.fail == 0) {
          // integrateSpectrum (src/integrator.cpp:730-743): the samples on
          // the grid of multiples of hs in (t0, t]
          double t = __dmul_rn(__dadd_rn(floor(__ddiv_rn(s0.t, hs)), 1.0), hs);
          const double nt = __dmul_rn(__dadd_rn(floor(__ddiv_rn(p.t, hs)), 1.0), hs);
          const double lim = __dsub_rn(nt, __ddiv_rn(hs, 2.0));
          while (t < lim) {
            double xx, xy, xz;
            noise_sample(P, Q, s0, t, xx, xy, xz);
            // goertzel_stage_1, goertzel_stage_2_vector's b and covMat::add_outer
            // (src/floquet.cpp:25-38, 107-120)
            const double nx = __dsub_rn(__dadd_rn(xx, __dmul_rn(c2, s1x)), s2x);
            const double ny = __dsub_rn(__dadd_rn(xy, __dmul_rn(c2, s1y)), s2y);
            const double nz = __dsub_rn(__dadd_rn(xz, __dmul_rn(c2, s1z)), s2z);
            s2x = s1x; s2y = s1y; s2z = s1z;
            s1x = nx; s1y = ny; s1z = nz;
            imx = __dadd_rn(imx, __dmul_rn(2.0, __dmul_rn(__dmul_rn(sn, s2x), xx)));
            imy = __dadd_rn(imy, __dmul_rn(2.0, __dmul_rn(__dmul_rn(sn, s2y), xy)));
            imz = __dadd_rn(imz, __dmul_rn(2.0, __dmul_rn(__dmul_rn(sn, s2z), xz)));
            t = __dadd_rn(t, hs);
            ++ns;
            if (((++guard) & 4095u) == 0u && past_deadline(dl)) hit = true;
            if (hit) break;
          }
        }
        if (p.stop) nan_fill(p);
        p.n_steps += 1;
        if (((++guard) & 255u) == 0u && past_deadline(dl)) hit = true;
      }
      hit = __any_sync(0xffffffffu, hit);
      if (!hit) {
        if (lane == 0) {
          store_state(a.s, i, p);
          if (window >= 0) a.s.w_done[i] = window + 1;
          sp.nsamp[i] = ns;
        }
        if (lane < kSpecFreqs) {
          const int64_t n = a.s.n;
          sp.s1[(int64_t)(lane * 3 + 0) * n + i] = s1x;
          sp.s1[(int64_t)(lane * 3 + 1) * n + i] = s1y;
          sp.s1[(int64_t)(lane * 3 + 2) * n + i] = s1z;
          sp.s2[(int64_t)(lane * 3 + 0) * n + i] = s2x;
          sp.s2[(int64_t)(lane * 3 + 1) * n + i] = s2y;
          sp.s2[(int64_t)(lane * 3 + 2) * n + i] = s2z;
          sp.im[(int64_t)(lane * 3 + 0) * n + i] = imx;
          sp.im[(int64_t)(lane * 3 + 1) * n + i] = imy;
          sp.im[(int64_t)(lane * 3 + 2) * n + i] = imz;
        }
      }
    }
  }
  if (hit && lane == 0) atomicExch(&a.status->deadline_hit, 1);
  if (a.count_work && lane == 0 && n_seg) atomicAdd(&a.status->segments, n_seg);
}

int launch_spectrum(const RunArgs& a, int window, double next_t, const SpecArgs& sp, void* stream) {
  if (a.s.n == 0) return 0;
  const int64_t threads = a.s.n * 32;
  const unsigned grid = (unsigned)((threads + kSpecBlock - 1) / kSpecBlock);
  if (a.any_gas)
    k_spectrum<true><<<grid, kSpecBlock, 0, (cudaStream_t)stream>>>(a, window, next_t, sp);
  else
    k_spectrum<false><<<grid, kSpecBlock, 0, (cudaStream_t)stream>>>(a, window, next_t, sp);
  return (int)cudaGetLastError();
}

}  // namespace st
