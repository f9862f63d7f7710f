"""Batched parameter sets (st_create_batch): one context holding sets of
different integrators, fields, walls, gas and run lengths, as in the
reference's parameter sweeps, where each set is an independent reference run
(seed_s = s * particles, so set s particle i is the reference's run with
seed_s and ipart i).

Every set of a batched run must agree with the oracle run of that set alone
(counts exact, spins to 1e-9, trajectory to 1e-7 as in the golden parity
tests), and bit for bit with a GPU context holding that set alone.  Gas-free
sets alone run the gas-free instantiation of the trajectory-ahead kernel, the
batched context (gas in some sets) the general one, so the bit-for-bit check
also covers that specialisation.
"""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st

pytestmark = pytest.mark.gpu

S_TOL = 1e-9
X_TOL = 1e-7


def sweep_sets(nsets=12, per=16):
    r = np.random.default_rng(3)
    sets = []
    for s in range(nsets):
        dop = s < nsets // 2
        tf = r.uniform(0.01, 0.05) if dop else r.uniform(1e-5, 5e-5)
        g = r.uniform(0.0, 1e-8, 9)
        o = st.make_options(numParticles=per, dist="M", T=0.4, gas_coll=(s % 3 != 0), gravity=True,
                            B0=(r.uniform(1e-6, 1e-5), 0.0, 0.0), Gx=g[0:3], Gy=g[3:6], Gz=g[6:9],
                            E=(0.0, 0.0, 75e5 if r.uniform() < 0.5 else -75e5), diffuse=r.uniform(0.0, 0.5),
                            yi=(0.0, 0.0, 1.0), tf=tf, ioutInt=tf / 2, integratorType=0 if dop else 1, seed=s * per)
        sets.append(st.derive(o))
    # a set without particles in the middle: it takes no work and no index
    empty = st.make_options(numParticles=0, dist="M", T=0.4, gas_coll=True, tf=0.02, ioutInt=0.01, seed=99)
    sets.insert(nsets // 2, st.derive(empty))
    return sets


def close(a, b, tol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.where(both_nan, 0.0, np.abs(a - b) / np.maximum(1.0, np.abs(b)))
    return bool(np.all(d <= tol)) and not np.any(np.isnan(a) != np.isnan(b))


@pytest.mark.parametrize("kernel", [st.KERNEL_PERSISTENT, st.KERNEL_PLAIN], ids=["persistent", "plain"])
def test_batched_sets_match_the_oracle_and_single_set_runs(gpu, oracle, kernel):
    from _oracle import Options
    sets = sweep_sets()
    nw = max(st.num_windows(o) for o in sets)
    with st.Particles(sets) as p:
        p.init_particles()
        p.run_windows(0, nw, kernel)
        out = p.output_data()
        counters = p.counters()
    assert counters["dop_attempts"] > 0 and counters["rk45_attempts"] > 0
    first = 0
    for s, o in enumerate(sets):
        n = int(o.numParticles)
        got = {k: v[first:first + n] for k, v in out.items()}
        first += n
        if n == 0:
            continue
        _, ref = oracle.run_sample(Options.from_buffer_copy(bytes(o)), 0, n)
        for f in ("fail", "n_coll", "n_bounce", "n_steps"):
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"set {s} {f}")
        assert close(got["S"], ref["S"], S_TOL), f"set {s} S"
        for f in ("t", "pos", "v"):
            assert close(got[f], ref[f], X_TOL), f"set {s} {f}"
        with st.Particles(o) as q:
            q.init_particles()
            q.run_windows(0, st.num_windows(o), kernel)
            alone = q.output_data()
        for f in alone:
            np.testing.assert_array_equal(got[f], alone[f], err_msg=f"set {s} {f} (alone)")
