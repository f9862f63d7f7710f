"""GPU parity: the CUDA engine against the reference's own outputs.

Every golden case (tests/golden/*.bin, written by the reference CPU build) is
re-run on the GPU through the C ABI (st_main_analysis, both kernels) and
compared snapshot by snapshot:
  * failureState, n_coll, n_bounce, n_steps: bit-exact (the RNG draw stream
    and every trajectory decision must match);
  * t, pos, v: to 1e-7 relative.  The trajectory arithmetic is the
    reference's, operation for operation and without FMA, so it is
    bit-identical wherever CUDA's log / acos / cos / sin return the same double
    as libm.  Where they differ by an ulp (Marsaglia normals, diffuse angles),
    the wall-time root solve amplifies it: for a trajectory grazing the ceiling
    sqrt(vy^2 - 2 g (y - Ly/2)) has a near-zero argument, and a 1e-12 change in
    vy^2 moves the hit time by ~1e-8 s.  Measured deviations are <= 4e-9 m on
    these cases, with every count still exact;
  * spin S: |dS| <= 1e-9 per component (FP64, rtol 1e-12), the bar the
    reference's own integrator test uses.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES
import spintrack as st
from spintrack.formats import header_equal, read_format_a

pytestmark = pytest.mark.gpu

S_TOL = 1e-9
T_TOL = 1e-7
X_TOL = 1e-7


def compare(got, ref, s_tol=S_TOL):
    assert got.shape == ref.shape
    for f in ("fail", "n_coll", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f)
    for f, tol in (("t", T_TOL), ("pos", X_TOL), ("v", X_TOL)):
        a, b = got[f], ref[f]
        assert np.array_equal(np.isnan(a), np.isnan(b)), f
        m = ~np.isnan(b)
        scale = np.maximum(1.0, np.abs(b[m]))
        assert np.all(np.abs(a[m] - b[m]) <= tol * scale), (f, np.max(np.abs(a[m] - b[m])))
    a, b = got["S"], ref["S"]
    assert np.array_equal(np.isnan(a), np.isnan(b))
    m = ~np.isnan(b)
    err = np.max(np.abs(a[m] - b[m])) if m.any() else 0.0
    assert err <= s_tol, err
    return err


@pytest.mark.parametrize("kernel", [st.KERNEL_PLAIN, st.KERNEL_PERSISTENT], ids=["plain", "persistent"])
@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_case(gpu, tmp_path, case, kernel):
    opt = st.parse_params(GOLDEN / f"{case}.params")
    out = tmp_path / "gpu.bin"
    st.main_analysis(opt, out, kernel=kernel)
    a, b = out.read_bytes(), (GOLDEN / f"{case}.bin").read_bytes()
    assert len(a) == len(b)
    assert header_equal(a, b)
    _, got = read_format_a(out)
    _, ref = read_format_a(GOLDEN / f"{case}.bin")
    compare(got, ref)


def test_plain_and_persistent_agree(gpu, tmp_path):
    """Both kernels run the same device step code: identical outputs."""
    opt = st.parse_params(GOLDEN / "m04_gas.params")
    st.main_analysis(opt, tmp_path / "a.bin", kernel=st.KERNEL_PLAIN)
    st.main_analysis(opt, tmp_path / "b.bin", kernel=st.KERNEL_PERSISTENT)
    _, a = read_format_a(tmp_path / "a.bin")
    _, b = read_format_a(tmp_path / "b.bin")
    for f in a.dtype.names:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


def test_run_until_matches_window_driver(gpu):
    """runSimulation(nextTOut) called per window equals the window driver."""
    opt = st.derive(st.parse_params(GOLDEN / "c1_precess.params"))
    with st.Particles(opt) as p, st.Particles(opt) as q:
        p.init_particles()
        q.init_particles()
        for w in range(st.num_windows(opt)):
            p.run_simulation((w + 1.0) * opt.ioutInt)
        q.run_windows(0, st.num_windows(opt), st.KERNEL_PERSISTENT)
        a, b = p.output_data(), q.output_data()
    for f in a:
        np.testing.assert_array_equal(a[f], b[f], err_msg=f)


@pytest.mark.parametrize("case", ["m04_gas", "c_gas", "m42_diffuse", "nmax", "rk45", "traj", "pulse"])
def test_every_persistent_variant_matches_plain(gpu, case):
    """Every launch variant of the batched engine (the flattened kernel, the
    trajectory-ahead kernel with each ring size and top-up rule, its
    warp-specialised form and the three-lanes-per-particle kernel) runs the
    same device arithmetic as the plain kernel: outputs must be identical."""
    from spintrack import _capi
    opt = st.derive(st.parse_params(GOLDEN / f"{case}.params"))
    nwin = st.num_windows(opt)
    with st.Particles(opt) as p:
        p.init_particles()
        p.run_windows(0, nwin, st.KERNEL_PLAIN)
        ref = p.output_data()
    for v in range(_capi.load().st_launch_variant_count()):
        with st.Particles(opt) as p:
            if st.variant_name(v).startswith("tpp3") and opt.integratorType == 1:
                with pytest.raises(st.SpinTrackError):  # the three-lane step is DOP853's
                    p.set_launch_config(v, 0)
                continue
            p.set_launch_config(v, 0)
            p.init_particles()
            p.run_windows(0, nwin, st.KERNEL_PERSISTENT)
            got = p.output_data()
        for f in ref:
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f"variant {v} field {f}")
