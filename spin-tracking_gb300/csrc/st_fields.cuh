// Field hooks: the user-editable magnetic field model.
//
// These replace the reference's compile-time hooks (src/integrator.cpp:40-46):
//     __PREPROC__ coords pulse(const _PREC t, _PREC a, _PREC w)  -> {0, 0, a cos(w t)}
//     __PREPROC__ coords grad(coords& pos, const options OPT)     -> {pos.Gx, pos.Gy, pos.Gz}
// and keep their "edit this file and rebuild" model.  The spin sees
//     B(t) = pulse(t) + B0 + cross(v, E) / c^2 + grad(pos(t))
// along each ballistic segment (src/integrator.cpp:63-70).
//
// Fast path: with ST_GRAD_IS_LINEAR the kernels never evaluate st_grad per
// Runge-Kutta stage.  Because pos(tau) = p0 + v0 tau + (g/2) tau^2 y_hat is a
// polynomial in the time tau since the segment start, a linear grad gives
//     grad(pos(tau)) = grad(p0) + tau grad(v0) + tau^2 (g/2) grad(y_hat),
// so the per-segment setup calls st_grad three times and each stage costs two
// FMAs per component.  After editing st_grad into anything that is not linear
// in pos, set ST_GRAD_IS_LINEAR to 0: every stage then evaluates the hook.
// Likewise ST_PULSE_IS_Z_COS selects the built-in a*cos(w t) z pulse; set it to
// 0 after editing st_pulse.
//
// ST_TRAJ_CORRECTLY_ROUNDED 1 (the default) makes the trajectory's log, acos,
// cos and sin the correctly rounded ones of st_crmath.cuh, equal to the host
// C library's results wherever those are correctly rounded, instead of
// CUDA's (within an ulp; on 0.3% of gas-clock and 14-23% of reflection
// arguments not the host's).  Gas-collision and diffuse-wall trajectories
// then stay bit-exact with the CPU reference far longer: CUDA's functions
// swap a bounce within 0.1 s on a diffuse-0.94 configuration and diverge
// after 3 s on the reference's own params.txt.  The cost: ~7% of the
// throughput at diffuse 0.1, ~24% on a gas-heavy parameter sweep.  Set it
// to 0 for CUDA's functions.
#pragma once

#include "st_internal.h"

#ifndef ST_GRAD_IS_LINEAR
#define ST_GRAD_IS_LINEAR 1
#endif
#ifndef ST_PULSE_IS_Z_COS
#define ST_PULSE_IS_Z_COS 1
#endif
#ifndef ST_TRAJ_CORRECTLY_ROUNDED
#define ST_TRAJ_CORRECTLY_ROUNDED 1
#endif

namespace st {

struct Vec3 {
  double x, y, z;
};

// grad(pos): field of the linear gradient tensor, B_i = dot(pos, G_i).
__host__ __device__ inline Vec3 st_grad(const Vec3& pos, const SetParams& P) {
  Vec3 r;
  r.x = pos.x * P.Gx[0] + pos.y * P.Gx[1] + pos.z * P.Gx[2];
  r.y = pos.x * P.Gy[0] + pos.y * P.Gy[1] + pos.z * P.Gy[2];
  r.z = pos.x * P.Gz[0] + pos.y * P.Gz[1] + pos.z * P.Gz[2];
  return r;
}

// pulse(t): the dressing / pi-pulse field, along z with angular frequency w.
__host__ __device__ inline Vec3 st_pulse(double t, const SetParams& P) {
  Vec3 r;
  r.x = 0.0;
  r.y = 0.0;
  r.z = P.a * cos(P.w * t);
  return r;
}

}  // namespace st
