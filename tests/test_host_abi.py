"""Host-side logic of the C ABI, checked without a GPU: the library loads and
exports every declared entry point; options defaults, params parsing, window
count and the format-'A' writer agree with the oracle (and so with the
reference); unsupported options are rejected before any device work."""
from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, REPO
from spintrack import _capi
from spintrack._capi import Options, StateView, Vec3


def declared_functions() -> list[str]:
    names = []
    for h in (REPO / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"\b(st_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol(stlib):
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(stlib, n)]
    assert not missing, missing


def test_options_layout(stlib):
    assert stlib.st_options_size() == 440 == ctypes.sizeof(Options)


def test_defaults_equal_oracle(stlib, oracle):
    a = Options()
    stlib.st_options_default(ctypes.byref(a))
    assert bytes(a) == bytes(oracle.default_options())


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_parse_params_equals_oracle(stlib, oracle, case):
    a = Options()
    assert stlib.st_parse_params(str(GOLDEN / f"{case}.params").encode(), ctypes.byref(a)) == 0
    stlib.st_derive(ctypes.byref(a))
    b = oracle.parse_file(GOLDEN / f"{case}.params", derive=True)
    assert bytes(a) == bytes(b)
    # the header the reference wrote carries the same options image
    from spintrack.formats import header_equal
    assert header_equal(bytes(a), (GOLDEN / f"{case}.bin").read_bytes()[:440])


def test_parse_line_behaviour(stlib, oracle):
    o = Options()
    stlib.st_options_default(ctypes.byref(o))
    assert stlib.st_parse_line(ctypes.byref(o), b"tf, 2.5") == 0 and o.tf == 2.5
    assert stlib.st_parse_line(ctypes.byref(o), b"  B0 , 1e-6,2e-6 , 3e-6 ") == 0
    assert (o.B0.x, o.B0.y, o.B0.z) == (1e-6, 2e-6, 3e-6)
    # unrecognised keys are ignored (reported as 1), like the reference
    assert stlib.st_parse_line(ctypes.byref(o), b"output, a") == 1
    # fewer than two fields: "Misunderstood input line"
    assert stlib.st_parse_line(ctypes.byref(o), b"tf") == _capi.ST_ERR_ARG
    # a vector key needs three numbers; a number must parse
    assert stlib.st_parse_line(ctypes.byref(o), b"L, 1, 2") == _capi.ST_ERR_ARG
    assert stlib.st_parse_line(ctypes.byref(o), b"tf, abc") == _capi.ST_ERR_ARG
    # boolalpha semantics: "True" -> true, "1" -> false
    assert stlib.st_parse_line(ctypes.byref(o), b"gravity, True") == 0 and o.gravity
    assert stlib.st_parse_line(ctypes.byref(o), b"gravity, 1") == 0 and not o.gravity
    # stoi semantics: "1e7" parses as 1; a negative seed wraps to unsigned
    assert stlib.st_parse_line(ctypes.byref(o), b"nmax, 1e7") == 0 and o.nmax == 1
    assert stlib.st_parse_line(ctypes.byref(o), b"seed, -3") == 0 and o.seed == 2 ** 32 - 3
    assert stlib.st_parse_line(ctypes.byref(o), b"dist, Maxwell") == 0 and o.dist == b"M"
    # the oracle's parser agrees on all of the applied lines
    p = oracle.default_options()
    for line in ["tf, 2.5", "  B0 , 1e-6,2e-6 , 3e-6 ", "gravity, 1", "nmax, 1e7", "seed, -3", "dist, Maxwell"]:
        oracle.parse_line(p, line)
    assert bytes(p) == bytes(o)


def test_missing_params_file_keeps_defaults(stlib, tmp_path):
    o = Options()
    assert stlib.st_parse_params(str(tmp_path / "nope.txt").encode(), ctypes.byref(o)) == _capi.ST_ERR_IO
    d = Options()
    stlib.st_options_default(ctypes.byref(d))
    assert bytes(o) == bytes(d)


@pytest.mark.parametrize("tf,t0,iout,n", [(10, 0, 0.05, 200), (100, 0, 0.5, 200), (0.2, 0, 0.05, 4),
                                          (1, 0, 0.3, 3), (0.1, 0.5, 0.05, 0)])
def test_num_windows(stlib, tf, t0, iout, n):
    o = Options()
    stlib.st_options_default(ctypes.byref(o))
    o.tf, o.t0, o.ioutInt = tf, t0, iout
    assert stlib.st_num_windows(ctypes.byref(o)) == n


def test_writer_layout(stlib, tmp_path):
    """st_write_header + st_write_snapshot produce format 'A' byte for byte."""
    libc = ctypes.CDLL(None)
    libc.fopen.restype = ctypes.c_void_p
    libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    libc.fclose.argtypes = [ctypes.c_void_p]
    n = 5
    rng = np.random.default_rng(1)
    t = rng.random(n)
    pos, v, S = rng.random((n, 3)), rng.random((n, 3)), rng.random((n, 3))
    fail = np.array([0, 1, -1, 4, 0], np.int32)
    nc, nb, ns = (rng.integers(0, 1 << 40, n, dtype=np.uint64) for _ in range(3))
    P = lambda a, typ: a.ctypes.data_as(ctypes.POINTER(typ))  # noqa: E731
    view = StateView(P(t, ctypes.c_double), P(pos, Vec3), P(v, Vec3), P(S, Vec3), P(fail, ctypes.c_int32),
                     P(nc, ctypes.c_uint64), P(nb, ctypes.c_uint64), P(ns, ctypes.c_uint64))
    o = Options()
    stlib.st_options_default(ctypes.byref(o))
    o.numParticles = n
    path = tmp_path / "w.bin"
    f = libc.fopen(str(path).encode(), b"wb")
    assert stlib.st_write_header(ctypes.c_void_p(f), ctypes.byref(o)) == 0
    assert stlib.st_write_snapshot(ctypes.c_void_p(f), n, ctypes.byref(view)) == 0
    libc.fclose(ctypes.c_void_p(f))
    expect = bytes(o) + t.tobytes() + pos.tobytes() + v.tobytes() + S.tobytes() + fail.tobytes() + \
        nc.tobytes() + nb.tobytes() + ns.tobytes()
    assert path.read_bytes() == expect
    from spintrack.formats import read_format_a
    o2, snaps = read_format_a(path)
    assert len(snaps) == 1 and np.array_equal(snaps[0]["n_steps"], ns) and np.array_equal(snaps[0]["S"], S)


# integratorType 6 with the default w = 0: no Floquet period for its spectrum
@pytest.mark.parametrize("field,value,code", [("integratorType", 6, _capi.ST_ERR_ARG),
                                              ("dist", b"X", _capi.ST_ERR_UNSUPPORTED),
                                              ("ioutInt", 0.0, _capi.ST_ERR_ARG),
                                              ("numParticles", -1, _capi.ST_ERR_ARG)])
def test_create_rejects_before_device_work(stlib, field, value, code):
    o = Options()
    stlib.st_options_default(ctypes.byref(o))
    setattr(o, field, value)
    ctx = ctypes.c_void_p()
    assert stlib.st_create(ctypes.byref(o), 0, ctypes.byref(ctx)) == code
    assert not ctx.value
    assert stlib.st_last_error()


@pytest.mark.parametrize("name", ["out.h5", "OUT.HDF5", "run.Hdf5"])
def test_main_analysis_refuses_hdf5_names_before_device_work(stlib, tmp_path, name):
    """createLogger picks HDF5 by extension; a reference build without HDF5
    throws for such a name, and so does st_main_analysis (before any GPU call)."""
    o = Options()
    stlib.st_options_default(ctypes.byref(o))
    path = tmp_path / name
    assert stlib.st_main_analysis(ctypes.byref(o), str(path).encode(), 0, 1, None) == _capi.ST_ERR_UNSUPPORTED
    assert b"HDF5" in stlib.st_last_error()
    assert not path.exists()


def _random_params(rng):
    """A well-formed params file over random keys, formats and values."""
    scal = ["tf", "t0", "ioutInt", "rtol", "atol", "h", "hmax", "hmin", "T", "V", "m", "gamma", "diffuse",
            "maxPosStep", "a", "w", "beta", "safe", "fac1", "fac2", "uround"]
    ints = ["numParticles", "numPerGPUBlock", "seed", "nmax", "integratorType", "iout"]
    bools = ["gas_coll", "gravity", "fixedStepSize", "keepStepSize"]
    vecs = ["L", "B0", "E", "yi", "Gx", "Gy", "Gz"]
    def num():
        v = rng.normal() * 10.0 ** rng.integers(-12, 9)
        return rng.choice([repr(float(v)), f"{v:.6e}", f"{v:g}", f" {v:.3E} "])
    lines = []
    for _ in range(rng.integers(1, 25)):
        kind = rng.integers(0, 5)
        if kind == 0:
            lines.append(f"{rng.choice(scal)}, {num()}")
        elif kind == 1:
            lines.append(f"{rng.choice(ints)}, {int(rng.integers(-5, 100000))}")
        elif kind == 2:
            lines.append(f"{rng.choice(bools)}, {rng.choice(['true', 'false', 'True', 'FALSE', '0', '1'])}")
        elif kind == 3:
            lines.append(f" {rng.choice(vecs)} ,{num()}, {num()},{num()}")
        else:
            lines.append(f"dist, {rng.choice(['C', 'M', 'Maxwell', 'Constant'])}")
    return "\n".join(lines) + "\n"


def test_parse_params_equals_oracle_on_random_files(stlib, oracle, tmp_path):
    """The library's params parser and the oracle's (the reference's
    optionParser restated) give the same 440-byte options image on random
    well-formed files: keys in any order and repetition, numbers in every
    format stod accepts, booleans in boolalpha's cases, padded fields."""
    import numpy as np
    rng = np.random.default_rng(17)
    for k in range(200):
        path = tmp_path / f"r{k}.params"
        path.write_text(_random_params(rng))
        a = Options()
        assert stlib.st_parse_params(str(path).encode(), ctypes.byref(a)) == 0, path.read_text()
        b = oracle.parse_file(path, derive=False)
        assert bytes(a) == bytes(b), path.read_text()


@pytest.mark.parametrize("name", ["probe_spectrum", "probe_spectrum_m"])
def test_floquet_frequencies_match_reference(stlib, name):
    """The host library's floquet_diagonalize (the frequencies of the
    integratorType 6 aggregators) equals the reference build's bit for bit."""
    import spintrack as st
    from conftest import GOLDEN
    lines = (GOLDEN / f"{name}.txt").read_text().splitlines()
    want = [float.fromhex(x) for x in lines[1].split()[1:]]
    f, dt = st.floquet_frequencies(st.derive(st.parse_params(GOLDEN / f"{name}.params")))
    assert list(f) == want[:17] and dt == want[17]


def test_spectrum_needs_a_floquet_period(stlib):
    import spintrack as st
    opt = st.make_options(integratorType=6, w=0.0, a=5e-6)
    with pytest.raises(st.SpinTrackError):
        st.floquet_frequencies(opt)
