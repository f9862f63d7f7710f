"""Pin the oracle (oracle/spin_oracle.c) to the reference.

Every fixture under tests/golden/ was produced by the reference's own sources
(tests/golden/make_golden.py).  The oracle must reproduce them bit for bit on
this host (both built with -ffp-contract=off), and it must pass the
reference's own known-answer tests (tests/integrator_validation.cpp,
tests/particle_validation.cpp, tests/output_tests.cpp)."""
from __future__ import annotations

import ctypes
import math
import struct

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES
from _oracle import Rng, Vec3
from spintrack.formats import header_equal, read_format_a


def hexf(s: str) -> float:
    return float.fromhex(s)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_format_a_bit_exact(oracle, tmp_path, case):
    """mainAnalysis end to end: the whole output file equals the reference's."""
    opt = oracle.parse_file(GOLDEN / f"{case}.params")
    out = tmp_path / "o.bin"
    oracle.main_analysis(opt, out, threads=2)
    a, b = out.read_bytes(), (GOLDEN / f"{case}.bin").read_bytes()
    assert len(a) == len(b)
    assert header_equal(a, b)
    assert a[440:] == b[440:]


def _probe_lines(name):
    return [l.split() for l in (GOLDEN / name).read_text().splitlines() if l.strip()]


@pytest.mark.parametrize("dist", ["C", "M"])
def test_init_matches_reference(oracle, dist):
    """initParticlesCPU: positions, velocities, gas clock and RNG state."""
    params = GOLDEN / ("probe.params" if dist == "C" else "probe_m.params")
    opt = oracle.parse_file(params)
    p = oracle.alloc(opt.numParticles)
    oracle.L.or_init(ctypes.byref(opt), ctypes.byref(p), 0)
    for tok in _probe_lines(f"probe_init_{dist}.txt"):
        i = int(tok[1])
        vals = [hexf(x) for x in tok[2:9]]
        assert [p.pos[i].x, p.pos[i].y, p.pos[i].z] == vals[0:3]
        assert [p.v[i].x, p.v[i].y, p.v[i].z] == vals[3:6]
        assert p.next_gas[i] == vals[6]
        r = p.rng[i]
        assert [r.x, r.y, r.z, r.w] == [int(x) for x in tok[9:13]]
        assert int(r.has_spare) == int(tok[13])
        if r.has_spare:
            assert r.spare == hexf(tok[14])
    oracle.free(p)


def test_rng_draws_match_reference(oracle):
    """Raw xoshiro outputs and Marsaglia normals after init."""
    opt = oracle.parse_file(GOLDEN / "probe.params")
    p = oracle.alloc(opt.numParticles)
    oracle.L.or_init(ctypes.byref(opt), ctypes.byref(p), 0)
    for tok in _probe_lines("probe_draws.txt"):
        i = int(tok[1])
        k = (len(tok) - 2) // 2
        r = Rng.from_buffer_copy(bytes(p.rng[i]))
        raw = [oracle.L.or_xoshiro(ctypes.byref(r)) for _ in range(k)]
        assert raw == [int(x) for x in tok[2:2 + k]]
        nrm = [oracle.L.or_normal(ctypes.byref(r), 0.0, 1.0) for _ in range(k)]
        assert nrm == [hexf(x) for x in tok[2 + k:]]
    oracle.free(p)


def test_events_match_reference(oracle):
    """calc_next_collision_time + update_position_and_velocity + sanity_check
    sequences (gas, diffuse and specular events) for two parameter files."""
    blocks = (GOLDEN / "probe_events.txt").read_text().split("p 0\n")
    assert len(blocks) == 3
    for params, text in zip(["probe.params", "probe_m.params"], blocks[1:]):
        opt = oracle.parse_file(GOLDEN / params)
        p = oracle.alloc(opt.numParticles)
        oracle.L.or_init(ctypes.byref(opt), ctypes.byref(p), 0)
        i = 0
        nseg = 0
        for line in ("p 0\n" + text).splitlines():
            tok = line.split()
            if tok[0] == "p":
                i = int(tok[1])
                continue
            oracle.L.or_event(ctypes.byref(opt), ctypes.byref(p), i, opt.tf)
            ct, wh, stop, fail = tok[1], tok[2], int(tok[3]), int(tok[4])
            assert p.coll_type[i] == ct.encode()
            if wh != "-":
                assert p.wall_hit[i] == wh.encode()
            assert int(p.stop[i]) == stop and p.fail[i] == fail
            vals = [hexf(x) for x in tok[5:14]]
            assert p.t[i] == vals[1]
            assert [p.pos[i].x, p.pos[i].y, p.pos[i].z] == vals[2:5]
            assert [p.v[i].x, p.v[i].y, p.v[i].z] == vals[5:8]
            assert p.next_gas[i] == vals[8]
            assert p.rng[i].x == int(tok[14])
            nseg += 1
        assert nseg > 40
        oracle.free(p)


EXT_TYPE = {"magnus": 2, "rk45q": 3, "rkf45": 4, "rkf45q": 5}


@pytest.mark.parametrize("which", ["dop", "rk45", "magnus", "rk45q", "rkf45", "rkf45q"])
def test_segment_steppers_match_reference(oracle, which):
    """integrateDOP / integrateRK45 / integrateMagnusCFET /
    integrateRK45Quaternion / integrateRKF45 / integrateRKF45Quaternion over
    single ballistic segments, accepted steps and hmin failures alike."""
    fn = {"dop": oracle.L.or_integrate_dop, "rk45": oracle.L.or_integrate_rk45}.get(which, oracle.L.or_integrate_ext)
    for line in (GOLDEN / f"probe_{which}.txt").read_text().splitlines():
        lhs, rhs = line.split("|")
        a = lhs.split()
        opt = oracle.parse_file(GOLDEN / a[0])
        if which in EXT_TYPE:
            opt.integratorType = EXT_TYPE[which]
        v = [float(x) for x in a[1:]]
        y = Vec3(*v[2:5])
        p0 = Vec3(*v[5:8])
        v0 = Vec3(*v[8:11])
        h = ctypes.c_double(v[11])
        ret = fn(ctypes.byref(opt), v[0], v[1], ctypes.byref(y), ctypes.byref(p0), ctypes.byref(v0), ctypes.byref(h))
        r = rhs.split()
        assert ret == int(r[1])
        assert [y.x, y.y, y.z, h.value] == [hexf(x) for x in r[2:6]]


def test_free_precession_kat(oracle):
    """tests/integrator_validation.cpp:12-46: DOP853 free precession about x
    over [0.1, 1.2] s with rtol = atol = 1e-12 matches the analytic spin to 1e-9."""
    opt = oracle.default_options()
    opt.B0 = Vec3(3e-6, 0.0, 0.0)
    opt.E = Vec3(0.0, 0.0, 0.0)
    opt.gravity = False
    opt.rtol = opt.atol = 1e-12
    y = Vec3(0.0, 0.0, 1.0)
    z = Vec3(0.0, 0.0, 0.0)
    h = ctypes.c_double(1e-4)
    oracle.L.or_integrate_dop(ctypes.byref(opt), 0.1, 1.2, ctypes.byref(y), ctypes.byref(z), ctypes.byref(z),
                              ctypes.byref(h))
    ph = 3e-6 * opt.gamma * (1.2 - 0.1)
    assert abs(y.x) <= 1e-9
    assert abs(y.y - math.sin(ph)) <= 1e-9
    assert abs(y.z - math.cos(ph)) <= 1e-9


def test_maxwell_boltzmann_init_kat(oracle):
    """tests/particle_validation.cpp:14-42: loose Maxwell-Boltzmann moments of
    1e5 initial velocities (T = 0.4 K, m = 1e-26 kg)."""
    opt = oracle.default_options()
    opt.gravity = False
    opt.T = 0.4
    opt.m = 1e-26
    opt.dist = b"M"
    opt.numParticles = 100000
    k = 1.380649e-23
    opt.sqrtKT_m = math.sqrt(k * opt.T / opt.m)
    p = oracle.alloc(opt.numParticles)
    oracle.L.or_init(ctypes.byref(opt), ctypes.byref(p), 0)
    v = oracle.arrays(p)["v"]
    oracle.free(p)
    s = math.sqrt(k * opt.T / opt.m)
    assert np.all(np.abs(v.sum(0) / 1e5 / s) < 2e-2)
    assert abs(math.sqrt((v ** 2).sum() / 1e5) / math.sqrt(3 * k * opt.T / opt.m) - 1) < 2e-2


def test_interpolation_kat(oracle):
    """tests/particle_validation.cpp:44-80: ballistic interpolation with and
    without gravity."""
    opt = oracle.default_options()
    p_old, v_old = Vec3(1, 2, 3), Vec3(1, 2, 3)
    po, vo = Vec3(), Vec3()
    opt.gravity = False
    oracle.L.or_interpolate(ctypes.byref(opt), 1.0, 0.0, ctypes.byref(p_old), ctypes.byref(v_old), ctypes.byref(po),
                            ctypes.byref(vo))
    assert (po.x, po.y, po.z, vo.x, vo.y, vo.z) == (2, 4, 6, 1, 2, 3)
    opt.gravity = True
    oracle.L.or_interpolate(ctypes.byref(opt), 1.0, 0.0, ctypes.byref(p_old), ctypes.byref(v_old), ctypes.byref(po),
                            ctypes.byref(vo))
    g = -9.81
    assert abs(po.y - (2 + 2 + 0.5 * g)) <= 1e-9 and abs(vo.y - (2 + g)) <= 1e-9
    assert (po.x, po.z, vo.x, vo.z) == (2, 6, 1, 3)


def test_output_test_kat():
    """tests/output_tests.cpp:20-82 re-expressed on format 'A': snapshot times
    are i*ioutInt and the spin is free precession at every snapshot (1e-9)."""
    opt, snaps = read_format_a(GOLDEN / "output_test.bin")
    assert len(snaps) == 5
    for i, s in enumerate(snaps):
        assert np.all(np.abs(s["t"] - i * opt.ioutInt) <= 1e-9)
        ph = 3e-6 * opt.gamma * i * opt.ioutInt
        assert np.all(np.abs(s["S"][:, 0]) <= 1e-9)
        assert np.all(np.abs(s["S"][:, 1] - math.sin(ph)) <= 1e-9)
        assert np.all(np.abs(s["S"][:, 2] - math.cos(ph)) <= 1e-9)


def test_golden_cases_exercise_the_paths():
    """The fixture set covers gas collisions, diffuse bounces, failures and
    edge/corner stops, so bit-exactness above is meaningful."""
    seen = {"gas": 0, "fail": 0, "bounce": 0}
    for case in GOLDEN_CASES:
        _, s = read_format_a(GOLDEN / f"{case}.bin")
        if len(s) == 0:
            continue
        last = s[-1]
        seen["gas"] += int(last["n_coll"].sum())
        seen["bounce"] += int(last["n_bounce"].sum())
        seen["fail"] += int((last["fail"] != 0).sum())
    assert seen["gas"] > 100 and seen["bounce"] > 1000 and seen["fail"] > 0


def test_parser_matches_reference_on_random_files(oracle, tmp_path):
    """optionParser (the reference's own, through oracle/_ref/ref_probe) and the
    oracle's restatement give the same options image, derived fields
    included, on 100 random well-formed params files (keys in any order and
    repetition, every number format stod accepts, boolalpha cases)."""
    import subprocess
    from pathlib import Path
    import numpy as np
    from test_host_abi import _random_params
    probe = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_probe"
    if not probe.exists():
        pytest.skip("the reference build (oracle/_ref) is not present on this machine")
    rng = np.random.default_rng(29)
    for k in range(100):
        path = tmp_path / f"r{k}.params"
        path.write_text(_random_params(rng))
        out = subprocess.run([str(probe), "options", str(path)], capture_output=True, text=True, timeout=60).stdout
        ref = bytes.fromhex(out.strip().splitlines()[-1].split()[1])
        ours = bytes(oracle.parse_file(path, derive=True))
        assert header_equal(ours, ref), path.read_text()


def _check_events(oracle, params, text):
    """Replay the reference's event lines (ref_probe events) with the oracle."""
    opt = oracle.parse_file(params)
    p = oracle.alloc(opt.numParticles)
    try:
        oracle.L.or_init(ctypes.byref(opt), ctypes.byref(p), 0)
        i, nseg = 0, 0
        for line in text.splitlines():
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "p":
                i = int(tok[1])
                continue
            oracle.L.or_event(ctypes.byref(opt), ctypes.byref(p), i, opt.tf)
            assert p.coll_type[i] == tok[1].encode()
            if tok[2] != "-":
                assert p.wall_hit[i] == tok[2].encode()
            assert int(p.stop[i]) == int(tok[3]) and p.fail[i] == int(tok[4])
            vals = [hexf(x) for x in tok[5:14]]
            assert p.t[i] == vals[1]
            assert [p.pos[i].x, p.pos[i].y, p.pos[i].z] == vals[2:5]
            assert [p.v[i].x, p.v[i].y, p.v[i].z] == vals[5:8]
            assert p.next_gas[i] == vals[8]
            assert p.rng[i].x == int(tok[14])
            nseg += 1
        return nseg
    finally:
        oracle.free(p)


def test_events_match_reference_on_random_configurations(oracle, tmp_path):
    """Trajectory events of the reference (ref_probe events) and of the oracle,
    bit for bit, over 24 random configurations: box sizes, 'C' speeds and
    'M' temperatures, gas on and off, diffuse fractions from 0 to 1, gravity
    on and off, seeds."""
    import subprocess
    from pathlib import Path
    import numpy as np
    probe = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_probe"
    if not probe.exists():
        pytest.skip("the reference build (oracle/_ref) is not present on this machine")
    rng = np.random.default_rng(41)
    total = 0
    for k in range(24):
        L = rng.uniform(0.02, 0.5, 3)
        dist = rng.choice(["C", "M"])
        T = float(rng.choice([0.4, 1.0, 4.2]))
        gas = bool(rng.random() < 0.5) and T < 4.0  # at 4.2 K the gas clock is picoseconds
        text = (f"numParticles, 6\ndist, {dist}\nV, {rng.uniform(1, 10):.6g}\nT, {T}\n"
                f"gas_coll, {'true' if gas else 'false'}\ndiffuse, {rng.uniform(0, 1):.6g}\n"
                f"gravity, {'true' if rng.random() < 0.7 else 'false'}\nL, {L[0]:.6g}, {L[1]:.6g}, {L[2]:.6g}\n"
                f"yi, 0, 0, 1\ntf, 1\nioutInt, 0.5\nseed, {int(rng.integers(0, 2**31))}\n")
        params = tmp_path / f"e{k}.params"
        params.write_text(text)
        out = subprocess.run([str(probe), "events", str(params), "60"], capture_output=True, text=True,
                             timeout=120).stdout
        total += _check_events(oracle, params, out)
    assert total > 24 * 6 * 30


@pytest.mark.parametrize("which", ["dop", "rk45", "magnus", "rk45q", "rkf45", "rkf45q"])
def test_segment_steppers_match_reference_on_random_segments(oracle, tmp_path, which):
    """Every stepper over 30 random ballistic segments (start time, length,
    spin, position, velocity, initial step; with and without the dressing
    pulse and gravity), the reference's own integrator (ref_probe) against the
    oracle's, bit for bit: return code, spin and carried step."""
    import subprocess
    from pathlib import Path
    import numpy as np
    probe = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_probe"
    if not probe.exists():
        pytest.skip("the reference build (oracle/_ref) is not present on this machine")
    rtol = {"dop": "1e-12", "rk45": "1e-12", "magnus": "1e-12", "rk45q": "1e-10", "rkf45": "1e-3", "rkf45q": "1e-6"}
    itype = {"dop": 0, "rk45": 1, **EXT_TYPE}
    fn = {"dop": oracle.L.or_integrate_dop, "rk45": oracle.L.or_integrate_rk45}.get(which, oracle.L.or_integrate_ext)
    rng = np.random.default_rng(7 + itype[which])
    for k in range(30):
        pulse = rng.random() < 0.5
        g = rng.normal(0.0, 1e-9, 9)
        text = (f"rtol, {rtol[which]}\ngravity, {'true' if rng.random() < 0.7 else 'false'}\n"
                f"B0, {rng.uniform(1e-6, 5e-6):.6g}, {rng.normal(0, 1e-7):.6g}, 0\nE, 0, 0, 75e5\n"
                f"Gx, {g[0]:.6g}, {g[1]:.6g}, {g[2]:.6g}\nGy, {g[3]:.6g}, {g[4]:.6g}, {g[5]:.6g}\n"
                f"Gz, {g[6]:.6g}, {g[7]:.6g}, {g[8]:.6g}\n" + ("a, 5e-6\nw, 6283.185307179586\nhmax, 1e-4\n" if pulse else ""))
        params = tmp_path / f"s{k}.params"
        params.write_text(text)
        t0 = rng.uniform(0.0, 1.0)
        length = 10.0 ** rng.uniform(-5, -2) if which in ("rk45", "rk45q", "rkf45q") else 10.0 ** rng.uniform(-4, -1)
        y = rng.normal(size=3)
        y /= np.linalg.norm(y)
        f = lambda x: repr(float(x))  # noqa: E731
        args = [f(t0), f(t0 + length), *map(f, y), *map(f, rng.uniform(-0.05, 0.05, 3)),
                *map(f, rng.normal(0, 5, 3)), f(10.0 ** rng.uniform(-6, -3)), "0"]
        out = subprocess.run([str(probe), which, str(params), *args], capture_output=True, text=True,
                             timeout=120).stdout.split()
        opt = oracle.parse_file(params)
        opt.integratorType = itype[which]
        v = [float(a) for a in args]
        yy, p0, v0, h = Vec3(*v[2:5]), Vec3(*v[5:8]), Vec3(*v[8:11]), ctypes.c_double(v[11])
        ret = fn(ctypes.byref(opt), v[0], v[1], ctypes.byref(yy), ctypes.byref(p0), ctypes.byref(v0), ctypes.byref(h))
        assert ret == int(out[1]), (k, args)
        assert [yy.x, yy.y, yy.z, h.value] == [hexf(x) for x in out[2:6]], (k, args)


def test_init_and_draws_match_reference_on_random_configurations(oracle, tmp_path):
    """initParticlesCPU and the draws after it (raw xoshiro outputs, Marsaglia
    normals) for 20 random configurations: 'C' speeds (including 0, where
    the reference still draws the three normals) and 'M' temperatures, gas on
    and off, box sizes, seeds up to 2^32 - 1."""
    import subprocess
    from pathlib import Path
    import numpy as np
    probe = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_probe"
    if not probe.exists():
        pytest.skip("the reference build (oracle/_ref) is not present on this machine")
    rng = np.random.default_rng(61)
    for k in range(20):
        L = rng.uniform(0.02, 0.5, 3)
        V = 0.0 if k == 0 else float(rng.uniform(0.5, 10))
        seed = int(rng.integers(0, 2**32)) if k % 2 else int(rng.integers(0, 100))
        text = (f"numParticles, 7\ndist, {rng.choice(['C', 'M'])}\nV, {V!r}\nT, {rng.choice([0.4, 1.3, 4.2])}\n"
                f"gas_coll, {rng.choice(['true', 'false'])}\nL, {L[0]!r}, {L[1]!r}, {L[2]!r}\nseed, {seed}\n")
        params = tmp_path / f"i{k}.params"
        params.write_text(text)
        opt = oracle.parse_file(params)
        p = oracle.alloc(opt.numParticles)
        try:
            oracle.L.or_init(ctypes.byref(opt), ctypes.byref(p), 0)
            out = subprocess.run([str(probe), "init", str(params)], capture_output=True, text=True, timeout=60).stdout
            for tok in (l.split() for l in out.splitlines() if l.startswith("p ")):
                i = int(tok[1])
                vals = [hexf(x) for x in tok[2:9]]
                assert [p.pos[i].x, p.pos[i].y, p.pos[i].z] == vals[0:3], (k, text)
                assert [p.v[i].x, p.v[i].y, p.v[i].z] == vals[3:6], (k, text)
                assert p.next_gas[i] == vals[6]
                r = p.rng[i]
                assert [r.x, r.y, r.z, r.w] == [int(x) for x in tok[9:13]]
            out = subprocess.run([str(probe), "draws", str(params), "12"], capture_output=True, text=True,
                                 timeout=60).stdout
            for tok in (l.split() for l in out.splitlines() if l.startswith("p ")):
                i = int(tok[1])
                r = Rng.from_buffer_copy(bytes(p.rng[i]))
                raw = [oracle.L.or_xoshiro(ctypes.byref(r)) for _ in range(12)]
                assert raw == [int(x) for x in tok[2:14]], (k, text)
                nrm = [oracle.L.or_normal(ctypes.byref(r), 0.0, 1.0) for _ in range(12)]
                assert nrm == [hexf(x) for x in tok[14:26]], (k, text)
        finally:
            oracle.free(p)


def test_main_analysis_matches_reference_on_random_configurations(oracle, tmp_path):
    """mainAnalysis end to end on 12 random configurations (all six
    integrator types with tolerances each can meet, gas on and off, diffuse
    fractions, gravity on and off, the dressing pulse): the reference build's
    format-'A' file and the oracle's are equal bit for bit."""
    import subprocess
    from pathlib import Path
    import numpy as np
    exe = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "spintrack_ref"
    if not exe.exists():
        pytest.skip("the reference build (oracle/_ref) is not present on this machine")
    rtol = {0: "1e-12", 1: "1e-12", 2: "1e-12", 3: "1e-10", 4: "1e-3", 5: "1e-6"}
    tf = {0: 0.05, 1: 2e-4, 2: 0.05, 3: 0.01, 4: 0.004, 5: 4e-4}
    rng = np.random.default_rng(83)
    for k in range(12):
        it = k % 6
        L = rng.uniform(0.03, 0.4, 3)
        T = float(rng.choice([0.4, 0.7, 4.2]))
        g = rng.normal(0.0, 1e-9, 9)
        lines = [f"numParticles, 8", f"dist, {rng.choice(['C', 'M'])}", f"V, {float(rng.uniform(2, 8))!r}", f"T, {T}",
                 f"gas_coll, {'true' if (rng.random() < 0.5 and T < 4) else 'false'}",
                 f"diffuse, {float(rng.uniform(0, 1))!r}", f"gravity, {'true' if rng.random() < 0.7 else 'false'}",
                 f"L, {float(L[0])!r}, {float(L[1])!r}, {float(L[2])!r}",
                 f"B0, {float(rng.uniform(1e-6, 5e-6))!r}, 0, 0", "E, 0, 0, 75e5",
                 f"Gx, {float(g[0])!r}, {float(g[1])!r}, {float(g[2])!r}",
                 f"Gy, {float(g[3])!r}, {float(g[4])!r}, {float(g[5])!r}",
                 f"Gz, {float(g[6])!r}, {float(g[7])!r}, {float(g[8])!r}", "yi, 0, 0, 1", f"integratorType, {it}", f"rtol, {rtol[it]}",
                 f"tf, {tf[it]!r}", f"ioutInt, {tf[it] / 2!r}", f"seed, {int(rng.integers(0, 2**31))}"]
        if it in (0, 2) and rng.random() < 0.5:
            lines += ["a, 5e-6", "w, 6283.185307179586", "hmax, 1e-4"]
        params = tmp_path / f"m{k}.params"
        params.write_text("\n".join(lines) + "\n")
        ref_out, our_out = tmp_path / f"ref{k}.bin", tmp_path / f"ora{k}.bin"
        subprocess.run([str(exe), str(params), str(ref_out)], capture_output=True, text=True, timeout=300)
        oracle.main_analysis(oracle.parse_file(params), our_out, threads=2)
        a, b = our_out.read_bytes(), ref_out.read_bytes()
        assert len(a) == len(b) and header_equal(a, b), params.read_text()
        assert a[440:] == b[440:], params.read_text()


def spectrum_fixture(name):
    """A probe_spectrum*.txt fixture: noise arguments, the Floquet frequencies
    and dt, and per particle (samples, failure, bounces, collisions, s1, s2,
    imag_diag) after the first window."""
    lines = (GOLDEN / f"{name}.txt").read_text().splitlines()
    noise = [float(x) for x in lines[0].split()[1:]]
    f = [hexf(x) for x in lines[1].split()[1:]]
    parts = []
    for l in lines[2:]:
        tok = l.split()
        vals = np.array([hexf(x) for x in tok[6:]]).reshape(3, 17, 3)
        parts.append({"i": int(tok[1]), "n_samples": int(tok[2]), "fail": int(tok[3]), "n_bounce": int(tok[4]),
                      "n_coll": int(tok[5]), "s1": vals[0], "s2": vals[1], "imag": vals[2]})
    return noise, np.array(f[:17]), f[17], parts


@pytest.mark.parametrize("name", ["probe_spectrum", "probe_spectrum_m"])
def test_spectrum_matches_reference(oracle, name):
    """integratorType 6: floquet_diagonalize's frequencies and dt
    (src/integrator.cpp:824-867) and every particle's noise-spectrum
    aggregator (goertzel_stage_1/2_vector and covMat::add_outer,
    src/floquet.cpp:25-45, 107-120, fed by integrateSpectrum,
    src/integrator.cpp:730-743) after the first window, bit for bit."""
    noise, freq, dt, parts = spectrum_fixture(name)
    opt = oracle.parse_file(GOLDEN / f"{name}.params")
    opt.noiseAmplitudes.x, opt.noiseAmplitudes.y, opt.noiseAmplitudes.z = noise[0:3]
    opt.noiseFrequencies.x, opt.noiseFrequencies.y, opt.noiseFrequencies.z = noise[3:6]
    f, d = oracle.floquet_frequencies(opt)
    assert np.array_equal(f, freq) and d == dt
    opt.tf = opt.ioutInt  # the probe ran the first window
    out, spec = oracle.run_spectrum(opt, 0, opt.numParticles, threads=2)
    assert len(parts) == opt.numParticles
    for p in parts:
        i = p["i"]
        assert spec["n_samples"][i] == p["n_samples"] and out["fail"][i] == p["fail"]
        assert out["n_bounce"][i] == p["n_bounce"] and out["n_coll"][i] == p["n_coll"]
        for k in ("s1", "s2", "imag"):
            assert np.array_equal(spec[k][i], p[k]), (i, k)
    assert min(p["n_samples"] for p in parts) > 400
