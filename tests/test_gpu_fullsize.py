"""Parity at the headline size: 1,048,576 particles of the plain-at-scale
workload (MB at 4.2 K, diffuse 0.1, gravity, the full gradient tensor
G ~ N(0, 1e-9) drawn with numpy default_rng(0), E = (0, 0, 75e5),
B0 = (3e-6, 0, 0), DOP853 rtol 1e-12, gas off), shortened to one 0.05 s
window so the test runs in seconds.  The oracle cannot run a million
particles in a test, so:
  * samples at the start, middle and end of the index range agree with the
    oracle run of exactly those particles (counts exact, spins to 1e-9,
    trajectory to 1e-7, as in the golden parity tests);
  * a shard (particles [first, first + n) run alone with seed + first, the
    multi-GPU partition) equals the same particles of the full run bit for
    bit, at an offset past 2^19;
  * the plain and persistent kernels agree bit for bit on the whole run;
  * size-independent invariants hold for every particle: |S| = 1 to 1e-9
    (the steppers do not renormalise), positions inside the box, t = tf for
    particles still running, NaN state for stopped ones, failure codes from
    the reference's set.
"""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st

pytestmark = pytest.mark.gpu

N = 1 << 20
TF = 0.05


def headline_options(n=N, first=0):
    g = np.random.default_rng(0).normal(0.0, 1e-9, 9)
    return st.derive(st.make_options(
        numParticles=n, dist="M", T=4.2, diffuse=0.1, gas_coll=False, gravity=True, L=(0.07, 0.1, 0.4),
        B0=(3e-6, 0.0, 0.0), E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0), Gx=g[0:3], Gy=g[3:6], Gz=g[6:9], t0=0.0, tf=TF,
        ioutInt=TF, rtol=1e-12, atol=1e-12, h=1e-3, hmax=1.0, hmin=1e-8, integratorType=0,
        seed=(0 + first) & 0xFFFFFFFF))


@pytest.fixture(scope="module")
def full_run(gpu):
    opt = headline_options()
    out = {}
    for kernel in (st.KERNEL_PERSISTENT, st.KERNEL_PLAIN):
        with st.Particles(opt) as p:
            p.init_particles()
            assert p.run_windows(0, st.num_windows(opt), kernel) == 0
            out[kernel] = p.output_data()
    return opt, out


def close(a, b, tol):
    a, b = np.asarray(a, float), np.asarray(b, float)
    if not np.array_equal(np.isnan(a), np.isnan(b)):
        return False
    m = ~np.isnan(b)
    return bool(np.all(np.abs(a[m] - b[m]) <= tol * np.maximum(1.0, np.abs(b[m]))))


@pytest.mark.parametrize("first", [0, N // 2 - 24, N - 48])
def test_samples_match_the_oracle(full_run, oracle, first):
    from _oracle import Options
    opt, out = full_run
    got = {k: v[first:first + 48] for k, v in out[st.KERNEL_PERSISTENT].items()}
    _, ref = oracle.run_sample(Options.from_buffer_copy(bytes(opt)), first, 48)
    for f in ("fail", "n_coll", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f)
    assert close(got["S"], ref["S"], 1e-9)
    for f in ("t", "pos", "v"):
        assert close(got[f], ref[f], 1e-7), f


def test_a_shard_equals_its_slice_of_the_full_run(full_run):
    opt, out = full_run
    first, n = (1 << 19) + 12345, 4096
    shard = headline_options(n, first)
    with st.Particles(shard) as p:
        p.init_particles()
        p.run_windows(0, st.num_windows(shard), st.KERNEL_PERSISTENT)
        got = p.output_data()
    for f in got:
        np.testing.assert_array_equal(got[f], out[st.KERNEL_PERSISTENT][f][first:first + n], err_msg=f)


def test_kernels_agree_on_the_whole_run(full_run):
    _, out = full_run
    a, b = out[st.KERNEL_PERSISTENT], out[st.KERNEL_PLAIN]
    for f in a:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def test_invariants_of_every_particle(full_run):
    opt, out = full_run
    o = out[st.KERNEL_PERSISTENT]
    ok = ~np.isnan(o["t"])       # stopped particles (a failure code, or a diffuse edge/corner hit) are NaN
    assert ok.mean() > 0.99
    assert np.all(o["fail"][ok] == 0)
    assert set(np.unique(o["fail"])) <= {0, 1, 2, 3, 4, -1}
    np.testing.assert_allclose(np.linalg.norm(o["S"][ok], axis=1), 1.0, rtol=0, atol=1e-9)
    half = np.array([0.07, 0.1, 0.4]) / 2 + 1e-15
    assert np.all(np.abs(o["pos"][ok]) <= half)
    np.testing.assert_allclose(o["t"][ok], TF, rtol=0, atol=1e-15)
    assert np.all(np.isnan(o["S"][~ok]) & np.isnan(o["pos"][~ok]))
    assert np.all(o["n_steps"] >= o["n_bounce"])
    assert o["n_coll"].sum() == 0                              # gas off
