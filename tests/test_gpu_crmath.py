"""The trajectory's correctly rounded log, sin, cos and acos (st_crmath.cuh).

Against the committed vectors (tests/golden/crmath_vectors.txt: mpmath at 300
bits, rounded to the nearest double, over the argument ranges the trajectory
uses and their edges) and against the oracle's binary128 evaluation on 10^7
random arguments per function, every result must be the correctly rounded
one, for the fast paths with their rounding tests and for the accurate paths
alone; against the host C library (whose results the reference's
trajectories use) they must agree on all but a sliver of random arguments,
where CUDA's own functions differ on up to a fifth of them."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import GOLDEN
from spintrack import _capi

FNS = {"log": 0, "sin": 1, "cos": 2, "acos": 3}


def load_vectors():
    rows = [l.split() for l in (GOLDEN / "crmath_vectors.txt").read_text().splitlines() if l.strip()]
    out = {}
    for fn, x, y in rows:
        out.setdefault(fn, ([], []))
        out[fn][0].append(float.fromhex(x))
        out[fn][1].append(float.fromhex(y))
    return {k: (np.array(a), np.array(b)) for k, (a, b) in out.items()}


def libm():
    lib = ctypes.CDLL("libm.so.6")
    for fn in FNS:
        getattr(lib, fn).restype = ctypes.c_double
        getattr(lib, fn).argtypes = [ctypes.c_double]
    return lib


def test_vectors_are_what_the_host_library_returns_almost_always():
    """CPU check of the fixture: the host C library agrees with the correctly
    rounded values on nearly every vector (it is correctly rounded on all but
    ~0.1% of arguments)."""
    lib = libm()
    for fn, (x, y) in load_vectors().items():
        got = np.array([getattr(lib, fn)(float(v)) for v in x])
        assert np.mean(got != y) < 0.01, fn


def device_eval(fn, x):
    import torch
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    yd = torch.empty_like(xd)
    torch.cuda.synchronize()
    rc = _capi.load().st_crmath_eval(FNS[fn], ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()), len(x))
    assert rc == 0, _capi.load().st_last_error()
    return yd.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("fn", list(FNS))
def test_correctly_rounded_on_the_vectors(gpu, fn):
    x, y = load_vectors()[fn]
    got = device_eval(fn, x)
    bad = np.flatnonzero(got != y)
    assert bad.size == 0, [(x[i].hex(), got[i].hex(), y[i].hex()) for i in bad[:5]]


@pytest.mark.gpu
@pytest.mark.parametrize("fn", list(FNS))
def test_agree_with_the_host_library(gpu, fn):
    import torch
    rng = np.random.default_rng(5)
    u = rng.random(100000)
    x = {"log": 1.0 - u, "sin": 2.0 * np.pi * u, "cos": 2.0 * np.pi * u, "acos": np.sqrt(u)}[fn]
    lib = libm()
    host = np.array([getattr(lib, fn)(float(v)) for v in x])
    ours = device_eval(fn, x)
    cuda = getattr(torch, fn)(torch.tensor(x, dtype=torch.float64, device="cuda")).cpu().numpy()
    ulp = np.abs(ours.view(np.int64) - host.view(np.int64))
    assert ulp.max() <= 1
    assert np.mean(ours != host) < 0.005, (np.mean(ours != host), np.mean(cuda != host))


@pytest.mark.gpu
@pytest.mark.parametrize("fn", ["log", "sin", "cos", "acos", "sin_acos", "cos_acos"])
def test_correctly_rounded_on_ten_million_trajectory_arguments(gpu, oracle, fn):
    """Against the oracle's correctly rounded values (binary128 evaluation,
    one rounding; an algorithm independent of the device's double-double
    one) on 10^7 arguments formed as the trajectory forms them: 1 - u and the
    Marsaglia radius u^2 + v^2 for log, angles 2 pi u for sin and cos,
    sqrt(u) for acos and for the reflection's sin and cos of acos."""
    from test_oracle_math_modes import trajectory_arguments
    base = fn.split("_")[-1] if fn.endswith("acos") else fn
    x = trajectory_arguments(5_000_000 if fn == "log" else 10_000_000, seed=7)[base]
    if fn in ("sin_acos", "cos_acos"):
        code = 4 if fn == "sin_acos" else 5
        got = _device_eval_code(code, x)
        phi = oracle.math_eval("acos", x, correctly_rounded=True)
        want = oracle.math_eval(fn.split("_")[0], phi, correctly_rounded=True)
    else:
        got = device_eval(fn, x)
        want = oracle.math_eval(fn, x, correctly_rounded=True)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, (bad.size, [(x[i].hex(), got[i].hex(), want[i].hex()) for i in bad[:5]])


def _device_eval_code(code, x):
    import torch
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    yd = torch.empty_like(xd)
    torch.cuda.synchronize()
    rc = _capi.load().st_crmath_eval(code, ctypes.c_void_p(xd.data_ptr()), ctypes.c_void_p(yd.data_ptr()), len(x))
    assert rc == 0, _capi.load().st_last_error()
    return yd.cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("fn", ["log", "sin", "cos", "acos"])
def test_accurate_paths_alone_are_correctly_rounded(gpu, oracle, fn):
    """The accurate evaluations (the fallback of a fast result whose rounding
    is uncertain) on 10^6 trajectory arguments each."""
    from test_oracle_math_modes import trajectory_arguments
    x = trajectory_arguments(1_000_000, seed=9)[fn]
    got = _device_eval_code(8 + FNS[fn], x)
    want = oracle.math_eval(fn, x, correctly_rounded=True)
    bad = np.flatnonzero(got != want)
    assert bad.size == 0, (bad.size, [(x[i].hex(), got[i].hex(), want[i].hex()) for i in bad[:5]])
