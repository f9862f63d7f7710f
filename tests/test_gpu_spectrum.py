"""integratorType 6, the noise spectrum (src/integrator.cpp:724-743,
src/floquet.cpp:25-156), on the GPU against the oracle and the reference's
own aggregators.

The device kernel samples the noise field and runs the 17 Goertzel
recursions with the reference's operations in its order, and its trajectory
functions round correctly, so against the oracle in its correctly rounded
mode a run without test noise agrees bit for bit (the aggregators, samples,
counts); with test noise the device's sin(w t) enters and the aggregators
agree to 1e-9 of their largest magnitude.  Against the reference build's
fixtures (first window, probe_spectrum*.txt, made on another host's C
library) the same bars hold for counts and samples, with the aggregators to
1e-9.  Trajectories over several windows follow the plain kernel's bars, and
the covariance sum over particles equals a numpy restatement of
goertzel_stage_2 + get_covariance_spectrum over the oracle's aggregators."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN
import spintrack as st
from test_oracle_pin import spectrum_fixture

pytestmark = pytest.mark.gpu


def _options(name, windows=1):
    from _oracle import Options
    noise, _, _, _ = spectrum_fixture(name)
    opt = st.derive(st.parse_params(GOLDEN / f"{name}.params"))
    opt.noiseAmplitudes.x, opt.noiseAmplitudes.y, opt.noiseAmplitudes.z = noise[0:3]
    opt.noiseFrequencies.x, opt.noiseFrequencies.y, opt.noiseFrequencies.z = noise[3:6]
    opt.tf = opt.ioutInt * windows
    return opt, Options.from_buffer_copy(bytes(opt)), any(noise)


def _gpu(opt, kernel=st.KERNEL_PERSISTENT):
    with st.Particles(opt) as p:
        p.init_particles()
        assert p.run_windows(0, st.num_windows(opt), kernel) == 0
        return p.output_data(), p.spectrum_state(), p.covariance_spectrum(0)


def _close(a, b, rel):
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b))) <= rel * scale


@pytest.mark.parametrize("kernel", [st.KERNEL_PERSISTENT, st.KERNEL_PLAIN], ids=["persistent", "plain"])
@pytest.mark.parametrize("name", ["probe_spectrum", "probe_spectrum_m"])
def test_first_window_against_oracle_and_reference(gpu, oracle, name, kernel):
    opt, oo, noisy = _options(name)
    got, spec, _ = _gpu(opt, kernel)
    ref_out, ref = oracle.run_spectrum(oo, 0, opt.numParticles, math_mode=oracle.MATH_CR)
    for f in ("fail", "n_coll", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(got[f], ref_out[f], err_msg=f)
    np.testing.assert_array_equal(spec["n_samples"], ref["n_samples"])
    for k in ("s1", "s2", "imag"):
        if noisy:
            assert _close(spec[k], ref[k], 1e-9), k
        else:
            np.testing.assert_array_equal(spec[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(got["S"], ref_out["S"])  # type 6 integrates no spin
    # the reference build's aggregators (fixture)
    _, _, _, parts = spectrum_fixture(name)
    for p in parts:
        i = p["i"]
        assert spec["n_samples"][i] == p["n_samples"] and got["n_coll"][i] == p["n_coll"]
        assert got["n_bounce"][i] == p["n_bounce"] and got["fail"][i] == p["fail"]
        for k in ("s1", "s2", "imag"):
            assert _close(spec[k][i], p[k], 1e-9), (i, k)


def test_windows_restart_the_aggregators_and_trajectories_follow(gpu, oracle):
    """Three windows: the aggregators after the last hold only its samples, as
    the reference's window loop resets them; states, counts and spins as the
    oracle's; the covariance sum equals a numpy restatement."""
    opt, oo, _ = _options("probe_spectrum_m", windows=3)
    got, spec, (cov, nsum) = _gpu(opt)
    ref_out, ref = oracle.run_spectrum(oo, 0, opt.numParticles, math_mode=oracle.MATH_CR)
    for f in ("fail", "n_coll", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(got[f], ref_out[f], err_msg=f)
    for f in ("t", "pos", "v"):
        np.testing.assert_array_equal(got[f], ref_out[f], err_msg=f)
    for k in ("s1", "s2", "imag", "n_samples"):
        np.testing.assert_array_equal(spec[k], ref[k], err_msg=k)
    assert 400 < ref["n_samples"].min() and ref["n_samples"].max() < 600  # one window's samples
    f, dt = oracle.floquet_frequencies(oo)
    want = np.zeros((17, 3, 3), complex)
    for i in range(opt.numParticles):
        for k in range(17):
            ang = f[k] * dt
            c = (ref["s1"][i, k] - np.cos(ang) * ref["s2"][i, k]) + 1j * (np.sin(ang) * ref["s2"][i, k])
            m = np.outer(c, np.conj(c))
            m[np.diag_indices(3)] += -1j * ref["imag"][i, k]
            want[k] += m
    assert nsum == int(ref["n_samples"].sum())
    assert _close(cov, want, 1e-12)


def test_spectrum_contexts_refuse_mixing(gpu):
    opt, _, _ = _options("probe_spectrum_m")
    other = st.derive(st.parse_params(GOLDEN / "c1_precess.params"))
    with pytest.raises(st.SpinTrackError):
        st.Particles([opt, other])
