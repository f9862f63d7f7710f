"""The engine against the oracle on random configurations: box sizes, 'C'
speeds and 'M' temperatures, gas collisions on and off, diffuse fractions,
gravity on and off, gradient tensors, E and B0 fields, pulse on and off,
integrator types 0-5 with tolerances each can meet, seeds.  Each run
(64 particles, a few windows) through st_main_analysis on both kernels must
equal the oracle's format-'A' file: counts and failure codes exact,
trajectory to 1e-7 relative, spins to 1e-9."""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st
from spintrack.formats import header_equal, read_format_a

pytestmark = pytest.mark.gpu

RTOL = {0: 1e-12, 1: 1e-12, 2: 1e-12, 3: 1e-10, 4: 1e-3, 5: 1e-6}
TF = {0: 0.1, 1: 2e-4, 2: 0.1, 3: 0.02, 4: 0.005, 5: 5e-4}


def random_params(rng):
    it = int(rng.integers(0, 6))
    tf = TF[it]
    L = rng.uniform(0.03, 0.4, 3)
    T = float(rng.choice([0.4, 0.6, 4.2]))
    gas = bool(rng.random() < 0.5) and T < 4.0
    g = rng.normal(0.0, 1e-9, 9)
    lines = [f"numParticles, 64", f"dist, {rng.choice(['C', 'M'])}", f"V, {rng.uniform(2, 8):.6g}", f"T, {T}",
             f"gas_coll, {'true' if gas else 'false'}", f"diffuse, {rng.uniform(0, 1):.4g}",
             f"gravity, {'true' if rng.random() < 0.7 else 'false'}", f"L, {L[0]:.5g}, {L[1]:.5g}, {L[2]:.5g}",
             f"B0, {rng.uniform(1e-6, 5e-6):.6g}, 0, 0", f"E, 0, 0, {rng.choice([-1, 1]) * 75e5:g}",
             f"Gx, {g[0]:.6g}, {g[1]:.6g}, {g[2]:.6g}", f"Gy, {g[3]:.6g}, {g[4]:.6g}, {g[5]:.6g}",
             f"Gz, {g[6]:.6g}, {g[7]:.6g}, {g[8]:.6g}", "yi, 0, 0, 1", f"integratorType, {it}",
             f"rtol, {RTOL[it]:g}", f"tf, {tf:g}", f"ioutInt, {tf / 2:g}", f"seed, {int(rng.integers(0, 2**31))}"]
    if rng.random() < 0.3 and it in (0, 2):
        lines += ["a, 5e-6", "w, 6283.185307179586", "hmax, 1e-4"]
    return "\n".join(lines) + "\n"


@pytest.mark.parametrize("k", range(16))
def test_random_configuration_matches_the_oracle(gpu, oracle, tmp_path, k):
    rng = np.random.default_rng(1000 + k)
    params = tmp_path / "r.params"
    params.write_text(random_params(rng))
    cpu_out = tmp_path / "cpu.bin"
    oracle.main_analysis(oracle.parse_file(params), cpu_out, threads=0)
    _, ref = read_format_a(cpu_out)
    for kernel in (st.KERNEL_PERSISTENT, st.KERNEL_PLAIN):
        gpu_out = tmp_path / f"gpu{kernel}.bin"
        st.main_analysis(st.parse_params(params), gpu_out, kernel=kernel)
        assert header_equal(gpu_out.read_bytes(), cpu_out.read_bytes())
        _, got = read_format_a(gpu_out)
        assert got.shape == ref.shape
        for f in ("fail", "n_coll", "n_bounce", "n_steps"):
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"{f}\n{params.read_text()}")
        for f, tol in (("t", 1e-7), ("pos", 1e-7), ("v", 1e-7), ("S", 1e-9)):
            x, y = got[f], ref[f]
            assert np.array_equal(np.isnan(x), np.isnan(y)), f
            m = ~np.isnan(y)
            if m.any():
                err = np.max(np.abs(x[m] - y[m]) / np.maximum(1.0, np.abs(y[m])))
                assert err <= tol, (f, err, params.read_text())
