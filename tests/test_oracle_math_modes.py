"""The oracle's elementary-function modes (CPU).

The reference computes its trajectories' log, acos, sin and cos with the host
C library (gas clocks, Marsaglia normals, cosine-law reflections; the
reference's src/particle.cpp:89-119 and :309-328).  The oracle can also take
them correctly rounded (binary128 evaluation, one rounding) and audit every
call where the two differ.  These tests pin that mode to the committed
mpmath vectors, measure how often the host library is not correctly rounded
on the trajectory's arguments, and show on the reference's own params.txt that
a single such last-bit difference is enough to change a particle's event
counts seconds later: the mechanism behind the residual difference between
the reference and any implementation whose functions round correctly."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLDEN
from test_gpu_refparams import REFERENCE_DEFAULT

COUNTS = ("fail", "n_coll", "n_bounce", "n_steps")


def _vectors():
    out = {}
    for line in (GOLDEN / "crmath_vectors.txt").read_text().splitlines():
        if line.strip():
            fn, x, y = line.split()
            out.setdefault(fn, ([], []))
            out[fn][0].append(float.fromhex(x))
            out[fn][1].append(float.fromhex(y))
    return {k: (np.array(a), np.array(b)) for k, (a, b) in out.items()}


def test_correctly_rounded_mode_equals_the_mpmath_vectors(oracle):
    for fn, (x, y) in _vectors().items():
        got = oracle.math_eval(fn, x, correctly_rounded=True)
        bad = np.flatnonzero(got != y)
        assert bad.size == 0, (fn, [(x[i].hex(), got[i].hex(), y[i].hex()) for i in bad[:5]])


def trajectory_arguments(n, seed=1):
    """Arguments as the trajectory forms them: 1 - u (gas clocks), the
    Marsaglia radius s = u^2 + v^2 in (0, 1), acos(sqrt u), and angles 2 pi u."""
    r = np.random.default_rng(seed)
    u, v, w = r.random(n), r.random(n) * 2 - 1, r.random(n) * 2 - 1
    s = v * v + w * w
    return {"log": np.concatenate([1.0 - u, s[(s > 0) & (s < 1)]]), "acos": np.sqrt(u),
            "sin": u * 2.0 * np.pi, "cos": u * 2.0 * np.pi}


def test_host_library_misrounding_rate(oracle):
    """The host C library is within one ulp everywhere and correctly rounded
    on all but a fraction of a percent of the trajectory's arguments."""
    for fn, x in trajectory_arguments(1_000_000).items():
        cr = oracle.math_eval(fn, x, correctly_rounded=True)
        host = oracle.math_eval(fn, x, correctly_rounded=False)
        ulps = np.abs(cr.view(np.int64) - host.view(np.int64))
        rate = float(np.mean(ulps != 0))
        print(f"{fn}: host library not correctly rounded on {rate:.4%} of {x.size} arguments")
        assert ulps.max() <= 1, fn
        assert 0.0 < rate < 0.005, (fn, rate)


def _params_options(oracle, tmp_path, tf=10):
    p = tmp_path / "params.txt"
    p.write_text(REFERENCE_DEFAULT.replace("tf, 10", f"tf, {tf}"))
    return oracle.parse_file(p)


def test_default_mode_is_the_reference_after_audited_runs(oracle, tmp_path):
    opt = _params_options(oracle, tmp_path, tf=1)
    oracle.run_sample_audited(opt, 0, 8, threads=1, mode=oracle.MATH_CR)
    case = "m04_gas"  # gas collisions and diffuse walls: every function is called
    out = tmp_path / "o.bin"
    oracle.main_analysis(oracle.parse_file(GOLDEN / f"{case}.params"), out, threads=2)
    assert out.read_bytes()[440:] == (GOLDEN / f"{case}.bin").read_bytes()[440:]


def test_audit_counts_the_same_calls_in_both_modes_until_trajectories_part(oracle, tmp_path):
    """Over the first second no particle's counts part, and the audited runs
    (host library, correctly rounded) see the same misrounded calls."""
    opt = _params_options(oracle, tmp_path, tf=1)
    _, ref, a_ref = oracle.run_sample_audited(opt, 0, 64, mode=oracle.MATH_AUDIT)
    _, cr, a_cr = oracle.run_sample_audited(opt, 0, 64, mode=oracle.MATH_CR)
    for f in COUNTS:
        np.testing.assert_array_equal(ref[f], cr[f], err_msg=f)
    np.testing.assert_array_equal(a_ref["count"], a_cr["count"])
    np.testing.assert_array_equal(a_ref["first_arg"], a_cr["first_arg"])
    assert (a_ref["count"] > 0).mean() > 0.5  # most particles meet one within a second


def test_a_single_misrounded_call_changes_the_counts(oracle, tmp_path):
    """The reference's params.txt (gas at 0.4 K, diffuse 0.3) over 10 s:
    some particles end with other collision / bounce / segment counts when the
    functions round correctly, and for such a particle substituting the host
    library's result at ONE call of an otherwise correctly rounded run is
    enough to move its counts: the trajectories are chaotic at the last bit
    (an ulp in a gas clock or a reflected velocity grows through grazing
    parabolas until two events swap order)."""
    opt = _params_options(oracle, tmp_path)
    n = 64
    _, ref, _ = oracle.run_sample_audited(opt, 0, n, mode=oracle.MATH_AUDIT)
    _, cr, a_cr = oracle.run_sample_audited(opt, 0, n, mode=oracle.MATH_CR)
    parted = np.flatnonzero(~np.all([ref[f] == cr[f] for f in COUNTS], axis=0))
    print(f"{parted.size} of {n} particles end with other counts than the correctly rounded run")
    assert 0 < parted.size < n // 4
    explained = []
    for i in parted[:3]:
        for k in range(min(int(a_cr["count"][i]), 24)):
            _, one, a = oracle.run_sample_audited(opt, int(i), 1, mode=oracle.MATH_PICK, pick=np.array([k]))
            if any(one[f][0] != cr[f][i] for f in COUNTS):
                fn = oracle.FN_NAMES[int(a["first_fn"][0])]
                x = float(a["first_arg"][0])
                host = oracle.math_eval(fn, np.array([x]), False)[0]
                exact = oracle.math_eval(fn, np.array([x]), True)[0]
                explained.append((int(i), k, fn, x.hex(), host.hex(), exact.hex(), float(a["first_t"][0])))
                break
    for e in explained:
        print("particle %d: call %d, %s(%s) host %s correctly rounded %s at t = %.6g s" % e)
    assert explained, "no single-call substitution reproduced a change of counts"
