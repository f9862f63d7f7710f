"""Algorithmic FP64 work of the hot path, for the roofline.

Counts are of the engine's own arithmetic (st_device.cuh), FMA = 2 flops,
add / mul / div / sqrt = 1, transcendentals (cos of the pulse, log, exp) not
counted:

DOP853 attempt (dop_attempt):
  stage states  y + h * sum(a_ij k_j): 11 stages, 50 a_ij terms, 3 components
                (2n + 1 flops for n terms)                         333
  stage times   x - t0, fma(c_i, h, tau) x 10, tau + h             22
  field         Omega(tau) = o0 + tau (o1 + tau o2): 11 evaluations 132
  Bloch         y x Omega: 12 evaluations (11 stages + FSAL)       108
  8th-order sum and new state                                       51
  error rows    bhh (3 FMA) and er (8 terms), 3 components          63
  weights       atol + rtol max(|y|,|y1|), 1/sk (3 FMA refinement)  24
  norms         two weighted sums of squares                        16
  controller    deno, rsqrt(3 deno), err, err^(-1/8) (2 Newton),
                new h, end-of-segment test                          36
                                                          total    785
RK45 attempt (rk45_attempt): 6 field + Bloch evaluations (132), stage
  states (102), weights and error (62), controller and update (22)  318
Trajectory segment (traj_event + seg_setup + dop_begin): wall times (~20),
  ballistic move and speed (~30), checks (~5), field polynomial setup (~75),
  first derivative (21)                                             150
Integrator types 2-5 (ext_attempt; sincos of the rotations not counted):
  Magnus CFET8: 5 node fields (70) scaled by h (15), 16 exponents
    sum c_j h B_j (432), 16 Rodrigues rotations (40 each: 640), error and
    controller (34)                                                   1191
  RK45 with quaternions: 5 node fields (68), 9 rotation quaternions (117),
    7 quaternion products (196), 2 rotations q (0,S) q* (82), error and
    controller (34)                                                   497
  RKF45: as RK45                                                      318
  RKF45 with quaternions: 5 node fields (68), 5 rotation quaternions (65),
    4 products (112), 2 rotations (82), error and controller (34)     361
"""
FLOPS_PER_DOP_ATTEMPT = 785
FLOPS_PER_RK45_ATTEMPT = 318
FLOPS_PER_SEGMENT = 150
FLOPS_PER_EXT_ATTEMPT = {2: 1191, 3: 497, 4: 318, 5: 361}


def algorithmic_flops(counters: dict, ext_type: int | None = None) -> float:
    """FP64 work of a run's counted attempts; ext_type names the one type 2-5
    behind counters["ext_attempts"] (a run mixing several has no single
    figure for them: their attempts are then left out)."""
    ext = counters.get("ext_attempts", 0) * FLOPS_PER_EXT_ATTEMPT.get(ext_type, 0) if ext_type else 0
    return (counters["dop_attempts"] * FLOPS_PER_DOP_ATTEMPT + counters["rk45_attempts"] * FLOPS_PER_RK45_ATTEMPT
            + counters["segments"] * FLOPS_PER_SEGMENT + ext)
