"""Unwrapped precession phase accumulated on the device (turn counter per
particle, st_gather_phase, snapshot field `turns`, unwrapped ensemble
statistics).

With 1 ms windows the phase moves ~0.6 rad between snapshots (B0 = 3 uT,
611 rad/s), so numpy.unwrap of the snapshot phases is unambiguous: the
device's atan2(Sz, Sy) + 2 pi turns must equal it at every snapshot, for both
kernels.  A single 50 ms window (the phase turns ~5 times inside it) must end
with the same turns and phase.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import spintrack as st

pytestmark = pytest.mark.gpu


def phase_options(tf, ioutInt, n=256):
    g = np.random.default_rng(2).normal(0.0, 1e-9, 9)
    return st.derive(st.make_options(numParticles=n, dist="M", T=4.2, diffuse=0.1, gas_coll=False, gravity=True,
                                     Gx=g[0:3], Gy=g[3:6], Gz=g[6:9], E=(0.0, 0.0, 75e5), B0=(3e-6, 0.0, 0.0),
                                     yi=(0.0, 0.0, 1.0), tf=tf, ioutInt=ioutInt, seed=21))


def snapshot_phases(kernel, opt):
    import torch
    nw = st.num_windows(opt)
    with st.Particles(opt) as p:
        bb = p.snapshot_bytes()
        snap = torch.zeros(bb * nw, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        p.init_particles()
        p.run_windows(0, nw, kernel, snap.data_ptr())
        torch.cuda.synchronize()
        blocks = st.unpack_snapshots(snap.cpu().numpy(), opt.numParticles, p.snapshot_offsets(), bb, nw)
        ens = p.ensemble(0)
        phase = torch.empty(opt.numParticles, dtype=torch.float64, device="cuda")
        p.gather_phase(phase.data_ptr())
        torch.cuda.synchronize()
    return blocks, ens, phase.cpu().numpy()


@pytest.mark.parametrize("kernel", [st.KERNEL_PERSISTENT, st.KERNEL_PLAIN], ids=["persistent", "plain"])
def test_turns_unwrap_the_snapshot_phases(gpu, kernel):
    opt = phase_options(0.05, 0.001)
    assert st.num_windows(opt) == 50
    blocks, ens, phase = snapshot_phases(kernel, opt)
    ok = blocks["fail"][-1] == 0
    phi = np.arctan2(blocks["S_z"], blocks["S_y"])[:, ok]                      # [window, particle]
    phi0 = np.full((1, phi.shape[1]), math.atan2(1.0, 0.0))
    ref = np.unwrap(np.concatenate([phi0, phi]), axis=0)[1:]                 # continuous from t = 0
    turns_ref = np.rint((ref - phi) / (2 * np.pi)).astype(np.int64)
    np.testing.assert_array_equal(blocks["turns"][:, ok], turns_ref)
    assert np.abs(blocks["turns"][-1, ok]).max() >= 4                         # the phase did wrap, repeatedly
    np.testing.assert_allclose(phase[ok], ref[-1], rtol=0, atol=1e-12)
    # ensemble: unwrapped mean over the counted particles, and the frequency
    # shift, equal to the wrapped one when that does not alias
    assert abs(ens["phase_unwrapped_mean"] - ref[-1].mean()) <= 1e-12 * abs(ref[-1].mean())
    assert abs(ens["freq_shift_unwrapped"] - ens["freq_shift"]) <= 1e-6  # Hz; the wrapped analysis also clips at 5 sigma


def test_one_long_window_ends_with_the_same_turns(gpu):
    fine, _, _ = snapshot_phases(st.KERNEL_PERSISTENT, phase_options(0.05, 0.001))
    coarse, _, phase = snapshot_phases(st.KERNEL_PERSISTENT, phase_options(0.05, 0.05))
    ok = (fine["fail"][-1] == 0) & (coarse["fail"][-1] == 0)
    np.testing.assert_array_equal(coarse["turns"][-1, ok], fine["turns"][-1, ok])
    phi = np.arctan2(fine["S_z"][-1], fine["S_y"][-1]) + 2 * np.pi * fine["turns"][-1]
    # window ends cut segments differently, so the spins differ at the
    # integration tolerance, not by turns
    np.testing.assert_allclose(phase[ok], phi[ok], rtol=0, atol=1e-7)
