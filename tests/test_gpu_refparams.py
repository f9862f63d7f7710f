"""The reference's own default configuration (params.txt:1-19 of the
reference: 1,024 particles, 'C' at 5 m/s, gas collisions at 0.4 K, diffuse
0.3, gravity, B0 = (3e-6, 0, 0), E = (3e8, 0, 0) V/m, h = 5e-5, DOP853 at
rtol 1e-12, tf = 10 s in 20 windows; ~4,700 gas collisions per
particle-second, ~48 million segments), the GPU's format-'A' file against the
oracle's, at its full length.

The trajectory's log / acos / cos / sin are correctly rounded on the GPU.  The
reference takes them from the host C library, which is not correctly rounded
on ~0.1% of the trajectory's arguments (every particle meets such a call
within its first second), and the dynamics are chaotic at the last bit: an ulp
in a gas clock or a reflected velocity grows through ceiling-grazing
parabolas until a gas collision and a wall hit swap order, after which the
particle consumes its random stream differently.  So the bars are:
  * against the oracle with correctly rounded functions: every count of every
    particle at every one of the 21 snapshots is exact, the trajectory within
    1e-7 relative and the spins within 1e-9 -- the GPU reproduces the
    reference's algorithm exactly for the full 10 s;
  * against the reference's own results (the oracle with the host library):
    the first two seconds are exact in every count (trajectory 1e-7 and spins
    1e-9 for the first second); at 10 s the particles whose counts differ are exactly those where
    the two oracle runs differ (the residual is the host library's rounding,
    nothing of the GPU's), a measured fraction (~11% with glibc 2.39 on
    x86-64) bounded at 20%, and the ensemble (mean collision, bounce and
    segment counts, polarisation, mean precession phase) agrees within one
    standard error.
"""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st
from spintrack.formats import header_equal, read_format_a

pytestmark = pytest.mark.gpu

REFERENCE_DEFAULT = """dist, C
T, 0.4
gas_coll, true
diffuse, 0.3
rtol, 1.0e-12
gravity, true
B0, 3.0e-6, 0, 0
yi, 0, 0, 1
h, 0.00005
numParticles, 1024
numPerGPUBlock, 256
t0, 0.0
tf, 10
ioutInt, 0.5
integratorType, 0
output, a
a, 0
w, 6.28318531e3
E, 3e8, 0, 0
"""


COUNTS = ("fail", "n_coll", "n_bounce", "n_steps")
N = 1024


@pytest.fixture(scope="module")
def oracle_runs(oracle, tmp_path_factory):
    """The reference's results (oracle, host C library) as a format-'A' file,
    and the oracle's run with correctly rounded functions, snapshot by
    snapshot (both on every host core)."""
    d = tmp_path_factory.mktemp("refparams")
    params = d / "params.txt"
    params.write_text(REFERENCE_DEFAULT)
    cpu_out = d / "cpu.bin"
    oracle.main_analysis(oracle.parse_file(params), cpu_out, threads=0)
    _, cr, audit = oracle.run_sample_audited(oracle.parse_file(params), 0, N, threads=0, mode=oracle.MATH_CR,
                                             snapshots=True)
    return params, cpu_out, cr, audit


def _close(x, y, tol):
    assert np.array_equal(np.isnan(x), np.isnan(y))
    m = ~np.isnan(y)
    return float(np.max(np.abs(x[m] - y[m]) / np.maximum(1.0, np.abs(y[m])), initial=0.0)) <= tol


def _differing(a, b):
    return ~np.all([a[f] == b[f] for f in COUNTS], axis=0)


@pytest.mark.parametrize("kernel", [st.KERNEL_PERSISTENT, st.KERNEL_PLAIN], ids=["persistent", "plain"])
def test_reference_default_params_full_length(gpu, oracle_runs, tmp_path, kernel):
    params, cpu_out, cr, audit = oracle_runs
    gpu_out = tmp_path / "gpu.bin"
    st.main_analysis(st.parse_params(params), gpu_out, kernel=kernel)
    a, b = gpu_out.read_bytes(), cpu_out.read_bytes()
    assert len(a) == len(b) and header_equal(a, b)
    _, got = read_format_a(gpu_out)
    _, ref = read_format_a(cpu_out)
    assert len(got) == 21 == len(cr)

    # 1. the algorithm: exact against correctly rounded functions, every snapshot
    for k in range(len(cr)):
        bad = np.flatnonzero(_differing(got[k], cr[k]))
        assert bad.size == 0, (k, bad[:5].tolist())
        for f, tol in (("t", 1e-7), ("pos", 1e-7), ("v", 1e-7), ("S", 1e-9)):
            assert _close(got[k][f], cr[k][f], tol), (k, f)

    # 2. the reference's own results: every count exact for two seconds, the
    # trajectory and spins within the golden bars for the first second (later
    # the host library's last bits have grown past them in some particles)
    for k in range(5):  # t = 0 .. 2 s
        assert not _differing(got[k], ref[k]).any(), k
    for k in range(3):  # t = 0 .. 1 s
        for f, tol in (("t", 1e-7), ("pos", 1e-7), ("v", 1e-7), ("S", 1e-9)):
            assert _close(got[k][f], ref[k][f], tol), (k, f)
    # ... then apart only where the host library's rounding moved the reference
    g, r = got[-1], ref[-1]
    diff_gpu = _differing(g, r)
    diff_cr = _differing(cr[-1], r)
    first = [next((k for k in range(len(ref)) if _differing(got[k], ref[k])[i]), None)
             for i in np.flatnonzero(diff_gpu)]
    print(f"kernel {kernel}: {diff_gpu.sum()} of {N} particles ({diff_gpu.mean():.2%}) end with other counts "
          f"than the reference at 10 s; first differing snapshot of each: "
          f"{np.bincount([f for f in first if f is not None], minlength=21).tolist()}; "
          f"host-library calls not correctly rounded per particle: {audit['count'].mean():.1f}")
    np.testing.assert_array_equal(diff_gpu, diff_cr)
    assert diff_gpu.mean() <= 0.20, diff_gpu.mean()
    assert np.all(audit["count"][diff_gpu] > 0)

    n = len(r["t"])
    for f in ("n_coll", "n_bounce", "n_steps"):
        se = np.std(r[f].astype(float)) / np.sqrt(n)
        assert abs(g[f].mean() - r[f].mean()) <= se, (f, g[f].mean(), r[f].mean(), se)
    # polarisation |<S>| (standard error of the spins' projection on the mean
    # direction) and mean precession phase atan2(Sz, Sy) about B0
    ok_g, ok_r = ~np.isnan(g["S"][:, 0]), ~np.isnan(r["S"][:, 0])
    Sg, Sr = g["S"][ok_g], r["S"][ok_r]
    nr = Sr.mean(0) / np.linalg.norm(Sr.mean(0))
    se_p = (Sr @ nr).std() / np.sqrt(len(Sr))
    Pg, Pr = np.linalg.norm(Sg.mean(0)), np.linalg.norm(Sr.mean(0))
    assert abs(Pg - Pr) <= se_p, (Pg, Pr, se_p)
    phg, phr = np.arctan2(Sg[:, 2], Sg[:, 1]), np.arctan2(Sr[:, 2], Sr[:, 1])
    se_ph = phr.std() / np.sqrt(len(phr))
    assert abs(phg.mean() - phr.mean()) <= se_ph, (phg.mean(), phr.mean(), se_ph)
    assert ref["n_coll"][-1].sum() > 30_000_000
