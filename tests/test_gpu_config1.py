"""The reference's CPU-runnable plain case at its full size: 1,000 particles,
'C' at 5 m/s, specular walls, gravity, gas off, dBx/dz = 1e-9 T/m,
E = (0, 0, 75e5) V/m, B0 = (3e-6, 0, 0) T, DOP853 at rtol 1e-12, tf = 10 s in
200 windows of 0.05 s, with yi along B0 (as written) and across it
(yi = (0, 0, 1), where the spin precesses ~970 turns).  The GPU's format-'A'
file, all 201 snapshots, against the oracle's file for the same params (the
oracle reproduces the reference build bit for bit on the golden cases):
failure codes and counts exact, trajectory to 1e-7 relative, spins to 1e-9."""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st
from spintrack.formats import header_equal, read_format_a

pytestmark = pytest.mark.gpu

CONFIG1 = """numParticles, 1000
L, 0.07, 0.1, 0.4
B0, 3e-6, 0, 0
E, 0, 0, 75e5
gamma, -2.038e8
m, 1.20239e-26
dist, C
V, 5
gravity, true
diffuse, 0
gas_coll, false
Gx, 0, 0, 1e-9
yi, {yi}
t0, 0
tf, 10
integratorType, 0
rtol, 1e-12
atol, 1e-12
h, 1e-3
hmax, 1
hmin, 1e-8
ioutInt, 0.05
seed, 0
"""


@pytest.mark.parametrize("yi", ["1, 0, 0", "0, 0, 1"], ids=["yi-along-B0", "yi-across-B0"])
def test_config1_full_length_matches_the_oracle(gpu, oracle, tmp_path, yi):
    params = tmp_path / "config1.params"
    params.write_text(CONFIG1.format(yi=yi))
    gpu_out, cpu_out = tmp_path / "gpu.bin", tmp_path / "cpu.bin"
    st.main_analysis(st.parse_params(params), gpu_out, kernel=st.KERNEL_PERSISTENT)
    oracle.main_analysis(oracle.parse_file(params), cpu_out, threads=0)
    a, b = gpu_out.read_bytes(), cpu_out.read_bytes()
    assert len(a) == len(b) and header_equal(a, b)
    _, got = read_format_a(gpu_out)
    _, ref = read_format_a(cpu_out)
    assert len(got) == 201
    for f in ("fail", "n_coll", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f)
    for f, tol in (("t", 1e-7), ("pos", 1e-7), ("v", 1e-7), ("S", 1e-9)):
        x, y = got[f], ref[f]
        assert np.array_equal(np.isnan(x), np.isnan(y)), f
        m = ~np.isnan(y)
        err = np.max(np.abs(x[m] - y[m]) / np.maximum(1.0, np.abs(y[m])))
        assert err <= tol, (f, err)
    assert ref["n_bounce"][-1].sum() > 300 * 1000      # ~870 segments per particle in 10 s
