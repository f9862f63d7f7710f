"""The device time budget (st_set_deadline): a run that runs out of it stops
cleanly with ST_ERR_DEADLINE (lanes check %globaltimer, no kernel spins on
anything), the context stays usable, and calling again resumes from the
particles' last window-end checkpoints: the final state equals an
uninterrupted run's bit for bit, for both kernels, with DOP853 and with the
Magnus stepper (whose kernels are the integrator type 2-5 instantiations)."""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st
from spintrack._capi import ST_ERR_DEADLINE

pytestmark = pytest.mark.gpu


def deadline_options(integrator=0):
    return st.derive(st.make_options(numParticles=4096, dist="M", T=4.2, diffuse=0.1, gas_coll=False, gravity=True,
                                     Gx=(0.0, 0.0, 1e-9), E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0), tf=0.2,
                                     ioutInt=0.05, seed=17, integratorType=integrator))


@pytest.mark.parametrize("integrator", [0, 2], ids=["dop853", "magnus"])
@pytest.mark.parametrize("kernel", [st.KERNEL_PERSISTENT, st.KERNEL_PLAIN], ids=["persistent", "plain"])
def test_deadline_stops_and_the_next_call_resumes(gpu, kernel, integrator):
    opt = deadline_options(integrator)
    nw = st.num_windows(opt)
    with st.Particles(opt) as p:
        p.init_particles()
        assert p.run_windows(0, nw, kernel) == 0
        ref = p.output_data()
        p.init_particles()
        p.set_deadline(1e-4)  # far shorter than the run
        assert p.run_windows(0, nw, kernel) == ST_ERR_DEADLINE
        p.set_deadline(0.0)
        for _ in range(3):  # the next call finishes what is left
            if p.run_windows(0, nw, kernel) == 0:
                break
        got = p.output_data()
    for f in ref:
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f)


def test_deadline_in_the_warp_specialised_kernel(gpu):
    """The same with every warp-specialised variant (consumer warps stop at
    the budget, the producer warps wind down when their slots are given up)."""
    from spintrack import _capi
    opt = deadline_options(0)
    nw = st.num_windows(opt)
    with st.Particles(opt) as p:
        p.init_particles()
        assert p.run_windows(0, nw, st.KERNEL_PLAIN) == 0
        ref = p.output_data()
    split = [v for v in range(_capi.load().st_launch_variant_count()) if st.variant_name(v).startswith("split")]
    assert split
    for v in split:
        with st.Particles(opt) as p:
            p.set_launch_config(v, 0)
            p.init_particles()
            p.set_deadline(1e-4)
            assert p.run_windows(0, nw, st.KERNEL_PERSISTENT) == ST_ERR_DEADLINE
            p.set_deadline(0.0)
            for _ in range(3):
                if p.run_windows(0, nw, st.KERNEL_PERSISTENT) == 0:
                    break
            got = p.output_data()
        for f in ref:
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"variant {v} field {f}")
