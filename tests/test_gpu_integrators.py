"""Integrator types 2-5 on the GPU: Magnus CFET8 (2), RK45 with quaternions
(3), RKF45 (4) and RKF45 with quaternions (5) (src/integrator.cpp:339-722).

Their golden cases (magnus, rk45q, rkf45, rkf45q, rkf45_hmin, magnus_fixed)
run through both kernels in test_gpu_parity.py against the reference's own
files.  Here, against the oracle (whose steppers are pinned bit for bit to the
reference build):
  * one batch holding all six integrator types, the hmin (-1) and nmax (-2)
    failures of types 2-5, and gas collisions: every set agrees with the
    oracle run of that set alone (counts exact, spins to 1e-9, trajectory to
    1e-7, as in the golden parity tests), for both kernels;
  * a full-size Magnus run with the 1 kHz dressing pulse (16,384 particles):
    particles at both ends of the index range agree with the oracle;
  * every persistent-kernel variant gives the plain kernel's bits;
  * the steppers agree with each other on the same trajectories: Magnus and
    the quaternion RK45 track DOP853's spins (a check independent of the
    reference: a wrong rotation sense or composition order fails it at O(1)).
"""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st

pytestmark = pytest.mark.gpu

S_TOL = 1e-9
X_TOL = 1e-7
G = np.array([1.3e-9, -0.4e-9, 1e-9, 0.2e-9, 0.7e-9, -1.1e-9, -0.5e-9, 0.9e-9, 0.3e-9])


def close(a, b, tol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.where(both_nan, 0.0, np.abs(a - b) / np.maximum(1.0, np.abs(b)))
    return bool(np.all(d <= tol)) and not np.any(np.isnan(a) != np.isnan(b))


def check_against_oracle(oracle, o, got, first, n, what):
    from _oracle import Options
    _, ref = oracle.run_sample(Options.from_buffer_copy(bytes(o)), first, n)
    for f in ("fail", "n_coll", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f"{what} {f}")
    assert close(got["S"], ref["S"], S_TOL), f"{what} S"
    for f in ("t", "pos", "v"):
        assert close(got[f], ref[f], X_TOL), f"{what} {f}"


def mixed_sets(per=12):
    # (integratorType, rtol, simulated time, extra options)
    plan = [(0, 1e-12, 0.02, {}), (1, 1e-12, 4e-5, {}), (2, 1e-12, 0.02, {"a": 5e-6, "w": 6283.185307179586,
                                                                          "hmax": 1e-4}),
            (3, 1e-10, 0.01, {}), (4, 1e-3, 0.02, {}), (5, 1e-6, 0.02, {}),
            (4, 1e-12, 0.01, {}),                                   # RKF45 at rtol 1e-12: h < hmin, -1
            (2, 1e-12, 0.01, {"fixedStepSize": True, "h": 1e-4, "nmax": 40}),  # fixed step: nmax, -2
            (2, 1e-12, 0.02, {"gas": True}), (5, 1e-6, 0.02, {"gas": True})]
    sets = []
    for s, (it, rtol, tf, extra) in enumerate(plan):
        extra = dict(extra)
        gas = extra.pop("gas", False)
        o = st.make_options(numParticles=per, dist="M", T=0.4 if gas else 4.2, gas_coll=gas, diffuse=0.2,
                            gravity=True, Gx=G[0:3], Gy=G[3:6], Gz=G[6:9], E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0),
                            integratorType=it, rtol=rtol, tf=tf, ioutInt=tf / 2, seed=100 + s * per, **extra)
        sets.append(st.derive(o))
    return sets


@pytest.mark.parametrize("kernel", [st.KERNEL_PERSISTENT, st.KERNEL_PLAIN], ids=["persistent", "plain"])
def test_all_integrator_types_in_one_batch_match_the_oracle(gpu, oracle, kernel):
    sets = mixed_sets()
    nw = max(st.num_windows(o) for o in sets)
    with st.Particles(sets) as p:
        p.init_particles()
        p.run_windows(0, nw, kernel)
        out = p.output_data()
        counters = p.counters()
    assert counters["dop_attempts"] > 0 and counters["rk45_attempts"] > 0 and counters["ext_attempts"] > 0
    first = 0
    fails = set()
    for s, o in enumerate(sets):
        n = int(o.numParticles)
        got = {k: v[first:first + n] for k, v in out.items()}
        first += n
        check_against_oracle(oracle, o, got, 0, n, f"set {s} (type {o.integratorType})")
        fails |= set(int(x) for x in got["fail"])
    assert {-1, -2} <= fails  # both failure paths of types 2-5 were taken


def test_full_size_magnus_with_the_dressing_pulse(gpu, oracle):
    n = 16384
    o = st.derive(st.make_options(numParticles=n, dist="M", T=4.2, gas_coll=False, diffuse=0.2, gravity=True,
                                  Gx=G[0:3], Gy=G[3:6], Gz=G[6:9], E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0),
                                  integratorType=2, a=5e-6, w=6283.185307179586, hmax=1e-4, tf=0.02,
                                  ioutInt=0.01, seed=5))
    with st.Particles(o) as p:
        p.init_particles()
        p.run_windows(0, st.num_windows(o), st.KERNEL_PERSISTENT)
        out = p.output_data()
        counters = p.counters()
    assert counters["ext_attempts"] > n
    for first in (0, n - 48):
        got = {k: v[first:first + 48] for k, v in out.items()}
        check_against_oracle(oracle, o, got, first, 48, f"particles {first}..")
    assert np.all(np.isfinite(out["S"])) and np.all(out["fail"] == 0)
    np.testing.assert_allclose(np.linalg.norm(out["S"], axis=1), 1.0, atol=1e-10)  # rotations keep |S|


@pytest.mark.parametrize("case", ["magnus", "rk45q", "rkf45", "rkf45q", "rkf45_hmin", "magnus_fixed"])
def test_every_persistent_variant_matches_plain(gpu, case):
    from conftest import GOLDEN
    from spintrack import _capi
    opt = st.derive(st.parse_params(GOLDEN / f"{case}.params"))
    nwin = st.num_windows(opt)
    with st.Particles(opt) as p:
        p.init_particles()
        p.run_windows(0, nwin, st.KERNEL_PLAIN)
        ref = p.output_data()
    for v in range(_capi.load().st_launch_variant_count()):
        with st.Particles(opt) as p:
            if st.variant_name(v).startswith(("split", "tpp3")):  # built for integrator types 0 and 1 only
                with pytest.raises(st.SpinTrackError):
                    p.set_launch_config(v, 0)
                continue
            p.set_launch_config(v, 0)
            p.init_particles()
            p.run_windows(0, nwin, st.KERNEL_PERSISTENT)
            got = p.output_data()
        for f in ref:
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"variant {v} field {f}")


def test_steppers_agree_with_dop853(gpu):
    """Same particles, same trajectories: the spin after 50 ms by Magnus
    (rtol 1e-12) and by RK45 with quaternions (rtol 1e-10) equals DOP853's
    (rtol 1e-12) to the accuracy those tolerances give."""
    base = dict(numParticles=512, dist="M", T=4.2, gas_coll=False, diffuse=0.2, gravity=True, Gx=G[0:3],
                Gy=G[3:6], Gz=G[6:9], E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0), tf=0.05, ioutInt=0.05, seed=8)
    out = {}
    for it, rtol in ((0, 1e-12), (2, 1e-12), (3, 1e-10)):
        o = st.derive(st.make_options(integratorType=it, rtol=rtol, **base))
        with st.Particles(o) as p:
            p.init_particles()
            p.run_windows(0, st.num_windows(o), st.KERNEL_PERSISTENT)
            out[it] = p.output_data()
    for it in (2, 3):
        for f in ("n_steps", "n_bounce", "fail"):
            np.testing.assert_array_equal(out[it][f], out[0][f])
    assert np.max(np.abs(out[2]["S"] - out[0]["S"])) < 1e-8
    assert np.max(np.abs(out[3]["S"] - out[0]["S"])) < 1e-5
