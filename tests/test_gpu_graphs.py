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
