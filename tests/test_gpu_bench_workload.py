"""Parity of the benchmarked workload at the length it is benchmarked: the
plain-at-scale configuration as bench.py runs it (1,048,576 particles, MB at
4.2 K, diffuse 0.1, gravity, the full gradient tensor G ~ N(0, 1e-9) from
numpy default_rng(0), E = (0, 0, 75e5), B0 = (3e-6, 0, 0), DOP853 rtol 1e-12,
gas off, tf = 1 s in two 0.5 s windows).  Three blocks of 256 particles spread
over the 1M index range run as shards (a shard seeded with seed + first equals
its slice of the full run bit for bit, tests/test_gpu_fullsize.py) and are
compared at all three snapshots with
  * the oracle with correctly rounded elementary functions: every count exact,
    spins within 1e-9, trajectory within 1e-7 relative;
  * the reference's own results (the oracle with the host C library): the same
    bars for every particle that met no host-library result that was not
    correctly rounded (the audit), and exact counts for all but the particles
    whose counts that rounding moved (the oracle runs with the two kinds of
    functions differ there too) -- printed, and at most 2%.
"""
from __future__ import annotations

import numpy as np
import pytest

import spintrack as st

pytestmark = pytest.mark.gpu

COUNTS = ("fail", "n_coll", "n_bounce", "n_steps")
BLOCK = 256
FIRSTS = (0, (1 << 19) - BLOCK // 2, (1 << 20) - BLOCK)


def bench_options(n, first):
    import bench
    return bench.workload_options(n, 1.0, first)


def _close(x, y, tol):
    if not np.array_equal(np.isnan(x), np.isnan(y)):
        return False
    m = ~np.isnan(y)
    return float(np.max(np.abs(x[m] - y[m]) / np.maximum(1.0, np.abs(y[m])), initial=0.0)) <= tol


def _gpu_snapshots(opt):
    nw = st.num_windows(opt)
    out = []
    with st.Particles(opt) as p:
        p.init_particles()
        out.append(p.output_data())
        for w in range(nw):
            assert p.run_windows(w, w + 1, st.KERNEL_PERSISTENT) == 0
            out.append(p.output_data())
    return out


@pytest.mark.parametrize("first", FIRSTS)
def test_bench_workload_full_length(gpu, oracle, first):
    from _oracle import Options
    opt = bench_options(BLOCK, first)
    assert st.num_windows(opt) == 2
    got = _gpu_snapshots(opt)
    # the shard's options seed with seed + first, so the oracle runs it from local index 0
    o = Options.from_buffer_copy(bytes(opt))
    _, cr, _ = oracle.run_sample_audited(o, 0, BLOCK, mode=oracle.MATH_CR, snapshots=True)
    _, ref, audit = oracle.run_sample_audited(o, 0, BLOCK, mode=oracle.MATH_AUDIT, snapshots=True)
    assert len(got) == len(cr) == len(ref) == 3
    for k in range(3):
        for f in COUNTS:
            np.testing.assert_array_equal(got[k][f], cr[k][f], err_msg=f"snapshot {k} {f}")
        for f, tol in (("t", 1e-7), ("pos", 1e-7), ("v", 1e-7), ("S", 1e-9)):
            assert _close(got[k][f], cr[k][f], tol), (k, f)
    moved = ~np.all([got[-1][f] == ref[-1][f] for f in COUNTS], axis=0)
    moved_oracle = ~np.all([cr[-1][f] == ref[-1][f] for f in COUNTS], axis=0)
    print(f"particles [{first}, {first + BLOCK}): {moved.sum()} of {BLOCK} end with other counts than the "
          f"reference; {int((audit['count'] > 0).sum())} met a host-library call that was not correctly rounded")
    np.testing.assert_array_equal(moved, moved_oracle)
    assert np.all(audit["count"][moved] > 0)
    assert moved.mean() <= 0.02
    clean = audit["count"] == 0
    assert clean.sum() >= BLOCK // 4
    for k in range(3):
        for f, tol in (("t", 1e-7), ("pos", 1e-7), ("v", 1e-7), ("S", 1e-9)):
            assert _close(got[k][f][clean], ref[k][f][clean], tol), (k, f)
