"""st_run_windows as CUDA graphs: the first call with a given kernel, window
range and snapshot buffer captures its launches into a graph, later calls
replay it.  Replays must give bit-identical results to the captured run and to
per-window calls, for both kernels, snapshots included."""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st

pytestmark = pytest.mark.gpu


def graph_options(n=256):
    return st.derive(st.make_options(numParticles=n, dist="M", T=4.2, diffuse=0.3, gas_coll=False, gravity=True,
                                     Gx=(0.0, 0.0, 1e-9), E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0), tf=0.2,
                                     ioutInt=0.05, seed=9))


@pytest.mark.parametrize("kernel", [st.KERNEL_PLAIN, st.KERNEL_PERSISTENT], ids=["plain", "persistent"])
def test_graph_replay_matches_capture_and_per_window_calls(gpu, kernel):
    import torch
    opt = graph_options()
    nw = st.num_windows(opt)
    assert nw == 4
    with st.Particles(opt) as p:
        snap = torch.zeros(p.snapshot_bytes() * nw, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        runs = []
        for rep in range(3):
            p.init_particles()
            p.run_windows(0, nw, kernel, snap.data_ptr())
            c = p.counters()
            assert c["graph_launches"] == 1
            assert c["graph_captures"] == (1 if rep == 0 else 0)
            if kernel == st.KERNEL_PLAIN:
                assert c["kernel_launches"] == 2 * nw  # one step and one pack launch per window
            torch.cuda.synchronize()
            runs.append((p.output_data(), snap.cpu().numpy().copy()))
        # the same windows one call each (each its own graph)
        p.init_particles()
        for w in range(nw):
            p.run_windows(w, w + 1, kernel)
        single = p.output_data()
    for out, blob in runs[1:]:
        np.testing.assert_array_equal(blob, runs[0][1])
        for f in out:
            np.testing.assert_array_equal(out[f], runs[0][0][f], err_msg=f)
    for f in single:
        np.testing.assert_array_equal(single[f], runs[0][0][f], err_msg=f)


def test_graph_cache_follows_the_launch_configuration(gpu):
    """A new launch configuration is a new graph; returning to an old one
    replays the cached graph; results never change."""
    opt = graph_options(128)
    nw = st.num_windows(opt)
    with st.Particles(opt) as p:
        outs, caps = [], []
        for var in (8, 5, 8):
            p.set_launch_config(var, 0)
            p.init_particles()
            p.run_windows(0, nw, st.KERNEL_PERSISTENT)
            caps.append(p.counters()["graph_captures"])
            outs.append(p.output_data())
    assert caps == [1, 1, 0]
    for out in outs[1:]:
        for f in out:
            np.testing.assert_array_equal(out[f], outs[0][f], err_msg=f)


@pytest.mark.parametrize("kernel", [st.KERNEL_PLAIN, st.KERNEL_PERSISTENT], ids=["plain", "persistent"])
def test_set_params_keeps_or_drops_the_graphs(gpu, kernel):
    """st_set_params with new field values keeps the captured graph (the
    kernels read the parameter table from device memory); switching the set to
    the Magnus stepper with gas collisions drops it (the graph holds the
    kernel instantiation).  Either way the run equals a fresh context holding
    the new parameters, bit for bit."""
    base = graph_options()
    nw = st.num_windows(base)
    values = st.derive(st.make_options(numParticles=256, dist="M", T=4.2, diffuse=0.3, gas_coll=False, gravity=True,
                                       Gx=(0.0, 0.0, 2e-9), E=(0.0, 0.0, -75e5), B0=(5e-6, 0.0, 0.0),
                                       yi=(0.0, 0.0, 1.0), tf=0.2, ioutInt=0.05, seed=9))
    kernels = st.derive(st.make_options(numParticles=256, dist="M", T=0.4, diffuse=0.3, gas_coll=True, gravity=True,
                                        Gx=(0.0, 0.0, 1e-9), E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0), tf=0.2,
                                        ioutInt=0.05, seed=9, integratorType=2))

    def fresh(opt):
        with st.Particles(opt) as q:
            q.init_particles()
            q.run_windows(0, nw, kernel)
            return q.output_data()

    with st.Particles(base) as p:
        p.init_particles()
        p.run_windows(0, nw, kernel)
        assert p.counters()["graph_captures"] == 1
        for new, captures in ((values, 0), (kernels, 1)):
            p.set_params(new)
            p.init_particles()
            p.run_windows(0, nw, kernel)
            c = p.counters()
            assert c["graph_launches"] == 1 and c["graph_captures"] == captures
            got, ref = p.output_data(), fresh(new)
            for f in ref:
                np.testing.assert_array_equal(got[f], ref[f], err_msg=f)
        assert c["ext_attempts"] > 0 and got["n_coll"].sum() > 0
