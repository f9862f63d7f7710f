// Ensemble statistics of one parameter set at one snapshot, on the device:
// mean spin and polarisation, and the precession phase analysis of the
// reference's scripts (scripts/nedmSim.py:151-179 shiftDatapoints and
// benchmarks/CheckingFrequencyShiftFromEField.ipynb analyzeDataset):
//   phi = atan2(Sz, Sy) of every particle with failureState 0;
//   align: with `location` the left edge of the most populated of 1000
//          equal bins over [min phi, max phi] (numpy.histogram's binning),
//          phi <= location - pi gains 2 pi, phi >= location + pi loses 2 pi;
//   clip:  drop phi outside mean +- 5 std of the aligned set;
//   mean and population std of what is left, the mean wrapped to [-pi, pi];
//   frequency shift = wrap(mean - atan2(cos(w t), sin(w t))) / (2 pi t),
//          w = gamma |B0| sign(B0x).
// Also the mean and population std of the unwrapped phase atan2(Sz, Sy) +
// 2 pi turns over the same particles (no alignment needed).
// Sums are per-block partials combined by one thread in block order, so the
// result is the same on every call.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <stdint.h>

#include "st_internal.h"

namespace st {

namespace {
constexpr int kEnsBlock = 256;
constexpr int kEnsBins = kEnsHistBins;
constexpr double kPi = 3.141592653589793;

struct EnsView {
  const double *t, *Sx, *Sy, *Sz;
  const int32_t *fail, *turns;
  int64_t first, n;
};

__device__ __forceinline__ double unwrapped(double phi, int turns) { return fma(2.0 * kPi, (double)turns, phi); }

// ctl slots: the ENS_* indices of st_internal.h

__device__ __forceinline__ bool ens_phi(const EnsView& v, int64_t i, double& phi) {
  if (v.fail[i] != 0) return false;
  phi = atan2(v.Sz[i], v.Sy[i]);
  return !isnan(phi);
}

// numpy's aligned value (both tests on the unshifted phase)
__device__ __forceinline__ double ens_align(double phi, double loc) {
  double p = phi;
  if (phi <= __dsub_rn(loc, kPi)) p = __dadd_rn(p, 2.0 * kPi);
  if (phi >= __dadd_rn(loc, kPi)) p = __dsub_rn(p, 2.0 * kPi);
  return p;
}

// numpy.histogram bin of x for `bins` equal bins over [e0, e1]
__device__ __forceinline__ int ens_bin(double x, double e0, double e1) {
  const double denom = __dsub_rn(e1, e0);
  const double f = __dmul_rn(__ddiv_rn(__dsub_rn(x, e0), denom), (double)kEnsBins);
  int k = (int)f;
  if (k >= kEnsBins) k = kEnsBins - 1;
  if (k < 0) k = 0;
  const double step = __ddiv_rn(denom, (double)kEnsBins);
  const double lo = __dadd_rn(__dmul_rn((double)k, step), e0);
  const double hi = (k + 1 == kEnsBins) ? e1 : __dadd_rn(__dmul_rn((double)(k + 1), step), e0);
  if (x < lo) --k;
  else if (x >= hi && k != kEnsBins - 1) ++k;
  return k;
}

// Block sum of up to 6 values (fixed tree order); thread 0 writes part[blk * 8 + q].
__device__ void block_store(double* sh, double v[6], int nv, double* part, bool is_minmax) {
  const int t = threadIdx.x;
  for (int q = 0; q < nv; ++q) {
    sh[t] = v[q];
    __syncthreads();
    for (int s = kEnsBlock / 2; s > 0; s >>= 1) {
      if (t < s) {
        if (is_minmax && q == 4) sh[t] = fmin(sh[t], sh[t + s]);
        else if (is_minmax && q == 5) sh[t] = fmax(sh[t], sh[t + s]);
        else sh[t] = sh[t] + sh[t + s];
      }
      __syncthreads();
    }
    if (t == 0) part[blockIdx.x * 8 + q] = sh[0];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kEnsBlock) k_ens_pass(EnsView v, int pass, const double* ctl, double* part,
                                                        unsigned int* hist) {
  __shared__ double sh[kEnsBlock];
  __shared__ unsigned int hsh[kEnsBins];
  const int64_t stride = (int64_t)gridDim.x * kEnsBlock;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (pass == 0) {
    acc[4] = INFINITY;
    acc[5] = -INFINITY;
  }
  if (pass == 1)
    for (int k = threadIdx.x; k < kEnsBins; k += kEnsBlock) hsh[k] = 0u;
  __syncthreads();
  for (int64_t j = (int64_t)blockIdx.x * kEnsBlock + threadIdx.x; j < v.n; j += stride) {
    const int64_t i = v.first + j;
    double phi;
    if (!ens_phi(v, i, phi)) continue;
    if (pass == 0) {
      acc[0] += 1.0;
      acc[1] += v.Sx[i];
      acc[2] += v.Sy[i];
      acc[3] += v.Sz[i];
      acc[4] = fmin(acc[4], phi);
      acc[5] = fmax(acc[5], phi);
    } else if (pass == 1) {
      atomicAdd(&hsh[ens_bin(phi, ctl[ENS_EDGE0], ctl[ENS_EDGE1])], 1u);
    } else if (pass >= 6) {  // unwrapped phase: sum, then squared deviations
      const double u = unwrapped(phi, v.turns[i]);
      if (pass == 6) {
        acc[0] += 1.0;
        acc[1] += u;
      } else {
        const double d = u - ctl[ENS_UMEAN];
        acc[1] = fma(d, d, acc[1]);
      }
    } else {
      const double p = ens_align(phi, ctl[ENS_LOC]);
      if (pass >= 4) {  // numpy: shifted < mean - std * 5, shifted > mean + std * 5
        const double w5 = __dmul_rn(ctl[ENS_STD1], 5.0);
        if (p < __dsub_rn(ctl[ENS_MEAN1], w5) || p > __dadd_rn(ctl[ENS_MEAN1], w5)) continue;
      }
      const double m = (pass == 3) ? ctl[ENS_MEAN1] : ctl[ENS_MEAN2];
      if (pass == 2 || pass == 4) {
        acc[0] += 1.0;
        acc[1] += p;
      } else {
        const double d = p - m;
        acc[1] = fma(d, d, acc[1]);
      }
    }
  }
  if (pass == 1) {
    __syncthreads();
    for (int k = threadIdx.x; k < kEnsBins; k += kEnsBlock)
      if (hsh[k]) atomicAdd(&hist[k], hsh[k]);
    return;
  }
  block_store(sh, acc, pass == 0 ? 6 : 2, part, pass == 0);
}

__global__ void k_ens_finish(EnsView v, int pass, double* ctl, const double* part, int nblk,
                             const unsigned int* hist) {
  if (threadIdx.x != 0) return;
  if (pass == 0) {
    double c = 0.0, sx = 0.0, sy = 0.0, sz = 0.0, mn = INFINITY, mx = -INFINITY;
    for (int b = 0; b < nblk; ++b) {
      c += part[b * 8];
      sx += part[b * 8 + 1];
      sy += part[b * 8 + 2];
      sz += part[b * 8 + 3];
      mn = fmin(mn, part[b * 8 + 4]);
      mx = fmax(mx, part[b * 8 + 5]);
    }
    ctl[ENS_COUNT] = c;
    ctl[ENS_SX] = sx;
    ctl[ENS_SY] = sy;
    ctl[ENS_SZ] = sz;
    ctl[ENS_MIN] = mn;
    ctl[ENS_MAX] = mx;
    double e0 = mn, e1 = mx;
    if (e0 == e1) {
      e0 = e0 - 0.5;
      e1 = e1 + 0.5;
    }
    ctl[ENS_EDGE0] = e0;
    ctl[ENS_EDGE1] = e1;
    double t = __longlong_as_double(0x7ff8000000000000ll);
    for (int64_t j = 0; j < v.n; ++j) {  // time of the first particle that counts
      double phi;
      if (ens_phi(v, v.first + j, phi)) {
        t = v.t[v.first + j];
        break;
      }
    }
    ctl[ENS_T] = t;
  } else if (pass == 1) {
    int best = 0;
    for (int k = 1; k < kEnsBins; ++k)
      if (hist[k] > hist[best]) best = k;  // first maximum, as numpy.argmax
    const double e0 = ctl[ENS_EDGE0], e1 = ctl[ENS_EDGE1];
    ctl[ENS_LOC] = __dadd_rn(__dmul_rn((double)best, __ddiv_rn(__dsub_rn(e1, e0), (double)kEnsBins)), e0);
  } else {
    double c = 0.0, s = 0.0;
    for (int b = 0; b < nblk; ++b) {
      c += part[b * 8];
      s += part[b * 8 + 1];
    }
    if (pass == 2) {
      ctl[ENS_MEAN1] = s / c;
    } else if (pass == 3) {
      ctl[ENS_STD1] = sqrt(s / ctl[ENS_COUNT]);
    } else if (pass == 4) {
      ctl[ENS_KEPT] = c;
      ctl[ENS_MEAN2] = s / c;
    } else if (pass == 5) {
      ctl[ENS_STD2] = sqrt(s / ctl[ENS_KEPT]);
    } else if (pass == 6) {
      ctl[ENS_UMEAN] = s / c;
    } else {
      ctl[ENS_USTD] = sqrt(s / ctl[ENS_COUNT]);
    }
  }
}
}  // namespace

// Run the passes for particles [first, first + n) of the given arrays; ctl
// receives ensemble_ctl_count() doubles (slots of the enum above).
int ensemble_device(const double* t, const double* Sx, const double* Sy, const double* Sz, const int32_t* fail,
                    const int32_t* turns, int64_t first, int64_t n, double* ctl, double* part, unsigned int* hist,
                    int max_blocks, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  EnsView v{t, Sx, Sy, Sz, fail, turns, first, n};
  const int nblk = (int)std::min<int64_t>(max_blocks, std::max<int64_t>(1, (n + kEnsBlock - 1) / kEnsBlock));
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(unsigned int) * kEnsBins, s);
  if (e != cudaSuccess) return (int)e;
  for (int pass = 0; pass <= 7; ++pass) {
    k_ens_pass<<<nblk, kEnsBlock, 0, s>>>(v, pass, ctl, part, hist);
    k_ens_finish<<<1, 32, 0, s>>>(v, pass, ctl, part, nblk, hist);
  }
  return (int)cudaGetLastError();
}

int ensemble_ctl_count() { return ENS_USTD + 1; }

// ---------------------------------------------------------------- phase
namespace {
__global__ void k_gather_phase(const double* Sy, const double* Sz, const int32_t* turns, int64_t n, double* dst) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = unwrapped(atan2(Sz[i], Sy[i]), turns[i]);
}
}  // namespace

int launch_gather_phase(const double* Sy, const double* Sz, const int32_t* turns, int64_t n, double* dst,
                        void* stream) {
  if (n <= 0) return 0;
  k_gather_phase<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(Sy, Sz, turns, n, dst);
  return (int)cudaGetLastError();
}

}  // namespace st
