"""The discrete adjoint against finite differences, for DOP853 and for the
Magnus CFET8 stepper.

Loss L = sum_i W_i . S_i(final) with fixed random weights W.  The GPU
gradient (st_adjoint_record + st_adjoint_backward through the torch Function)
is compared with central finite differences of the ORACLE (the reference
algorithm on the CPU) run with its accepted step sequence frozen to that
of the unperturbed run, which is the derivative the discrete adjoint computes.
Bar: 1e-6 relative per parameter.  Steps: relative 1e-6 of |B0| for B0 (the
spec's step) and for the pulse; the gradient tensor and E make up only 1e-5 to
1e-4 of the field, so a 1e-6 relative step in them moves L by 1e-9 to 1e-8,
where the ~1e-13 of uncorrelated rounding in L dominates the difference
quotient at the 1e-5 level.  They use relative steps of 1e-2 (G, each entry)
and 1e-4 of |E| (E), which change the precession by < 1e-5 rad, so L stays
linear in them to < 1e-9 while the rounding floor drops below 1e-7.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import pytest

import spintrack as st
from spintrack.adjoint import NUM_THETA, THETA_NAMES, precession_phase, theta_of, track_spins, with_theta

pytestmark = pytest.mark.gpu


def adj_options(n=8, tf=0.1, pulse=False, seed=5, integrator=0):
    g = np.random.default_rng(3).normal(0.0, 1e-9, 9)
    kw = dict(numParticles=n, dist="M", T=4.2, diffuse=0.0, gas_coll=False, gravity=True, Gx=g[0:3], Gy=g[3:6],
              Gz=g[6:9], E=(0.0, 0.0, 75e5), B0=(3e-6, 0.0, 0.0), yi=(0.0, 0.0, 1.0), tf=tf, ioutInt=0.05, seed=seed,
              rtol=1e-12, atol=1e-12, h=1e-3, hmax=1.0, hmin=1e-8, integratorType=integrator)
    if pulse:
        kw.update(a=5e-6, w=2 * math.pi * 1000.0, hmax=1e-4)
    return st.derive(st.make_options(**kw))


def oracle_loss(oracle, opt, W, log, mode):
    """Run the oracle (single thread) with the step log in `mode`; return L."""
    from _oracle import Options
    o = Options.from_buffer_copy(bytes(opt))
    oracle.L.or_set_step_log(log.ctypes.data_as(ctypes.c_void_p), log.shape[0] // 2, mode)
    try:
        _, out = oracle.run_sample(o, 0, o.numParticles, threads=1)
    finally:
        oracle.L.or_set_step_log(None, 0, 0)
    return float((out["S"] * W).sum()), out


def frozen_fd(oracle, opt, W, pulse):
    log = np.zeros(2 * 4_000_000)
    L0, base = oracle_loss(oracle, opt, W, log, 1)
    th = np.array(theta_of(opt))
    fd = np.zeros(NUM_THETA)
    for k in range(NUM_THETA):
        if k >= 15 and not pulse:
            continue
        if k < 9:
            d = 1e-2 * abs(th[k])
        elif k < 12:
            d = 1e-6 * 3e-6
        elif k < 15:
            d = 1e-4 * 75e5
        elif k == 15:
            d = 1e-6 * 3e-6
        else:
            d = 1e-6 * abs(th[k]) if th[k] != 0.0 else 1e-3
        lp, _ = oracle_loss(oracle, with_theta(opt, th + d * np.eye(NUM_THETA)[k]), W, log, 2)
        lm, _ = oracle_loss(oracle, with_theta(opt, th - d * np.eye(NUM_THETA)[k]), W, log, 2)
        fd[k] = (lp - lm) / (2 * d)
    return fd, base


def gpu_grad(opt, W, pulse):
    import torch
    dev = torch.device("cuda", 0)
    eng = st.Particles(opt)
    theta = torch.tensor([theta_of(opt)], dtype=torch.float64, device=dev, requires_grad=True)
    S = track_spins(theta, eng, [opt], st.num_windows(opt), pulse=pulse)
    L = (S * torch.tensor(W, device=dev)).sum()
    L.backward()
    g = theta.grad.detach().cpu().numpy()[0]
    S_np = S.detach().cpu().numpy()
    eng.close()
    return g, S_np


@pytest.mark.parametrize("integrator", [0, 2], ids=["dop853", "magnus"])
@pytest.mark.parametrize("pulse", [False, True], ids=["static", "pulse"])
def test_adjoint_matches_frozen_step_fd(gpu, oracle, pulse, integrator):
    opt = adj_options(pulse=pulse, integrator=integrator)
    W = np.random.default_rng(11).normal(size=(opt.numParticles, 3))
    g, S = gpu_grad(opt, W, pulse)
    fd, base = frozen_fd(oracle, opt, W, pulse)
    # the record pass is the forward map: spins agree with the oracle
    assert np.max(np.abs(S - base["S"])) <= 1e-9
    rows = []
    bad = []
    for k in range(NUM_THETA):
        if k >= 15 and not pulse:
            continue
        tol = 1e-6 * abs(fd[k]) + 1e-14 * np.max(np.abs(fd))
        rows.append(f"{THETA_NAMES[k]:5s} adj={g[k]: .10e} fd={fd[k]: .10e} rel={abs(g[k]-fd[k])/max(abs(fd[k]),1e-300):.2e}")
        if abs(g[k] - fd[k]) > tol:
            bad.append(rows[-1])
    assert not bad, "\n".join(rows)


@pytest.mark.parametrize("integrator", [0, 2], ids=["dop853", "magnus"])
def test_record_pass_is_the_forward_map(gpu, integrator):
    """st_adjoint_record advances particles exactly as st_run_windows."""
    opt = adj_options(n=64, tf=0.2, integrator=integrator)
    nw = st.num_windows(opt)
    with st.Particles(opt) as p, st.Particles(opt) as q:
        p.init_particles()
        p.run_windows(0, nw, st.KERNEL_PERSISTENT)
        q.init_particles()
        q.adjoint_record(nw)
        a, b = p.output_data(), q.output_data()
    for f in a:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def test_ensemble_losses_backpropagate(gpu):
    """Polarisation and precession-phase losses through torch autograd: the
    gradient is the adjoint's per-particle dL/dS contracted by torch."""
    import torch
    opt = adj_options(n=32, tf=0.1)
    dev = torch.device("cuda", 0)
    eng = st.Particles(opt)
    theta = torch.tensor([theta_of(opt)], dtype=torch.float64, device=dev, requires_grad=True)
    S = track_spins(theta, eng, [opt], st.num_windows(opt))
    loss = S[:, 0].mean() + S[:, 1].mean() + precession_phase(S).mean()
    loss.backward()
    g1 = theta.grad.clone()
    # the same gradient from an explicit dL/dS through the raw entry points
    with torch.no_grad():
        w = torch.zeros_like(S)
        n = S.shape[0]
        w[:, 0] += 1.0 / n
        w[:, 1] += 1.0 / n
        r2 = S[:, 1] ** 2 + S[:, 2] ** 2
        w[:, 1] += -S[:, 2] / r2 / n
        w[:, 2] += S[:, 1] / r2 / n
    out = torch.empty(n, NUM_THETA, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    eng.adjoint_backward(w.contiguous().data_ptr(), out.data_ptr())
    g2 = out.sum(0)
    eng.close()
    assert torch.allclose(g1[0], g2, rtol=1e-12, atol=0.0)
    assert torch.all(torch.isfinite(g1))


def _grad_with_budget(p, nw, w, tape_bytes, every):
    import torch
    p.init_particles()
    p.adjoint_record(nw, tape_bytes=tape_bytes, windows_per_checkpoint=every)
    out = torch.empty(p.n, NUM_THETA, dtype=torch.float64, device=w.device)
    torch.cuda.synchronize()
    p.adjoint_backward(w.data_ptr(), out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy(), p.adjoint_stats()


@pytest.mark.parametrize("integrator", [0, 2], ids=["dop853", "magnus"])
def test_backward_is_independent_of_the_tape_budget(gpu, integrator):
    """The same gradients whether the record pass's tape fits (no replay), or
    window chunks are replayed from state checkpoints, or a single window is
    replayed in particle groups; final states identical in every case."""
    import torch
    opt = adj_options(n=16, tf=0.2, integrator=integrator)
    nw = st.num_windows(opt)
    assert nw == 4
    dev = torch.device("cuda", 0)
    w = torch.tensor(np.random.default_rng(2).normal(size=(16, 3)), dtype=torch.float64, device=dev)
    with st.Particles(opt) as p:
        g_res, s_res = _grad_with_budget(p, nw, w, 0, 1)
        S_res = p.output_data()["S"]
        assert s_res["resident"] == 1 and s_res["replays"] == 0 and s_res["checkpoints"] == 4
        used = s_res["tape_bytes_used"]
        g_chunk, s_chunk = _grad_with_budget(p, nw, w, used // 2, 1)
        assert s_chunk["resident"] == 0 and s_chunk["replays"] >= 2 and s_chunk["groups"] == 0
        np.testing.assert_array_equal(p.output_data()["S"], S_res)
        g_grp, s_grp = _grad_with_budget(p, nw, w, used // 16, 1)
        assert s_grp["groups"] >= 2
        np.testing.assert_array_equal(p.output_data()["S"], S_res)

        # a pool below one particle's tape over one checkpoint interval
        p.init_particles()
        p.adjoint_record(nw, tape_bytes=2 * 320 * 8, windows_per_checkpoint=4)
        out = torch.empty(16, NUM_THETA, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        with pytest.raises(st.SpinTrackError):
            p.adjoint_backward(w.data_ptr(), out.data_ptr())
    assert np.all(np.isfinite(g_res))
    np.testing.assert_array_equal(g_chunk, g_res)
    np.testing.assert_array_equal(g_grp, g_res)


@pytest.mark.parametrize("integrator", [0, 2], ids=["dop853", "magnus"])
def test_record_keeps_the_last_intervals_when_the_tape_does_not_fit(gpu, integrator):
    """A pool too small for the whole tape but large enough for its last
    checkpoint intervals: the record pass (in pieces: the first interval,
    the middle with the tape off, the tail) keeps them and the backward
    replays only the earlier ones; the gradients and the forward outputs equal
    the resident tape's bit for bit."""
    import torch
    opt = adj_options(n=256, tf=0.4, integrator=integrator)
    nw = st.num_windows(opt)
    assert nw == 8
    dev = torch.device("cuda", 0)
    w = torch.tensor(np.random.default_rng(3).normal(size=(256, 3)), dtype=torch.float64, device=dev)
    with st.Particles(opt) as p:
        g_res, s_res = _grad_with_budget(p, nw, w, 0, 1)
        S_res = p.output_data()["S"]
        assert s_res["resident"] == 1 and s_res["record_launches"] == 2  # first interval, then the rest appended
        used = s_res["tape_bytes_used"]
        tails = []
        for frac in (0.9, 0.75, 0.6, 0.45):
            g_tail, s_tail = _grad_with_budget(p, nw, w, int(used * frac), 1)
            np.testing.assert_array_equal(p.output_data()["S"], S_res)
            if 0 < s_tail["tail_from"] < s_tail["checkpoints"]:
                assert s_tail["resident"] == 0 and s_tail["replays"] >= 1 and s_tail["record_launches"] == 3
                tails.append((frac, s_tail["tail_from"], g_tail))
    print("kept tails (pool fraction, first kept interval):", [(f, k) for f, k, _ in tails])
    assert tails, "no pool size kept a tail"
    for _, _, g_tail in tails:
        np.testing.assert_array_equal(g_tail, g_res)


def overshoot_options():
    """One particle (index 2412 of a seed-0 run) in a 1 kHz dressing field
    with gas collisions at 0.4 K and hmax 1e-4: one of its segments is
    shorter than hmin, so the step controller steps hmin past the segment end
    and closes the segment with a negative step, as the reference does."""
    g = np.random.default_rng(0).normal(0.0, 1e-9, 9)
    return st.derive(st.make_options(numParticles=1, dist="M", T=0.4, diffuse=0.5, gas_coll=True, gravity=True,
                                     Gx=g[0:3], Gy=g[3:6], Gz=g[6:9], E=(0.0, 0.0, 75e5), B0=(3e-6, 0.0, 0.0),
                                     yi=(0.0, 0.0, 1.0), tf=0.2, ioutInt=0.2, seed=2412, rtol=1e-12, atol=1e-12,
                                     h=1e-3, hmax=1e-4, hmin=1e-8, a=5e-6, w=2 * math.pi * 1000.0))


def test_adjoint_through_an_hmin_overshoot(gpu, oracle):
    from _oracle import Options
    opt = overshoot_options()
    log = np.zeros(2 * 200_000)
    oracle.L.or_set_step_log(log.ctypes.data_as(ctypes.c_void_p), log.shape[0] // 2, 1)
    try:
        oracle.run_sample(Options.from_buffer_copy(bytes(opt)), 0, 1, threads=1)
        n = int(oracle.L.or_step_log_count())
    finally:
        oracle.L.or_set_step_log(None, 0, 0)
    assert n > 0 and np.any(log[0:2 * n:2] < 0.0)  # the case is exercised: a negative accepted step
    W = np.random.default_rng(5).normal(size=(1, 3))
    g, S = gpu_grad(opt, W, True)
    fd, base = frozen_fd(oracle, opt, W, True)
    assert np.max(np.abs(S - base["S"])) <= 1e-9
    bad = [f"{THETA_NAMES[k]} adj={g[k]:.10e} fd={fd[k]:.10e}" for k in range(NUM_THETA)
           if abs(g[k] - fd[k]) > 1e-6 * abs(fd[k]) + 1e-14 * np.max(np.abs(fd))]
    assert not bad, "\n".join(bad)


def test_multi_loss_backward_equals_single_loss_calls(gpu):
    """st_adjoint_backward_multi with three losses gives, bit for bit, the
    gradients of three single-loss backward calls, with the tape resident and
    with window-chunk replays, where one replay of each chunk serves all three
    losses (as many replays as one single-loss call)."""
    import torch
    opt = adj_options(n=16, tf=0.2)
    nw = st.num_windows(opt)
    W = torch.tensor(np.random.default_rng(8).normal(size=(3, 16, 3)), dtype=torch.float64, device="cuda")
    with st.Particles(opt) as p:
        used = None
        for resident in (True, False):
            budget = 0 if resident else used // 2
            p.init_particles()
            p.adjoint_record(nw, tape_bytes=budget, windows_per_checkpoint=1)
            if resident:
                used = p.adjoint_stats()["tape_bytes_used"]
            out_m = torch.empty(3, 16, NUM_THETA, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            p.adjoint_backward_multi(3, W.data_ptr(), out_m.data_ptr())
            torch.cuda.synchronize()
            rep_multi = p.adjoint_stats()["replays"]
            assert rep_multi == 0 if resident else rep_multi >= 2
            for l in range(3):
                out = torch.empty(16, NUM_THETA, dtype=torch.float64, device="cuda")
                wl = W[l].contiguous()
                torch.cuda.synchronize()
                p.adjoint_backward(wl.data_ptr(), out.data_ptr())
                torch.cuda.synchronize()
                assert torch.equal(out, out_m[l]), f"loss {l}, resident={resident}"
                assert p.adjoint_stats()["replays"] == rep_multi


def test_stopped_particles_get_zero_gradients(gpu):
    """Particles that fail (here: DOP853 over nmax attempts in a segment)
    contribute nothing; the others are unaffected by their presence."""
    import torch
    opt = adj_options(n=32, tf=0.1)
    opt.nmax = 10  # segments needing more attempts fail with code -1 (2 of these 32 particles)
    nw = st.num_windows(opt)
    with st.Particles(opt) as p:
        p.init_particles()
        p.adjoint_record(nw)
        fail = p.output_data()["fail"]
        w = torch.ones(32, 3, dtype=torch.float64, device="cuda")
        out = torch.empty(32, NUM_THETA, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        p.adjoint_backward(w.data_ptr(), out.data_ptr())
        g = out.cpu().numpy()
    stopped = fail != 0
    assert stopped.any() and (~stopped).any()
    assert np.all(g[stopped] == 0.0)
    assert np.all(np.isfinite(g[~stopped])) and np.any(g[~stopped] != 0.0)
