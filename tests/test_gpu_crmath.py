"""The trajectory's correctly rounded log, sin, cos and acos (st_crmath.cuh).

Against the committed vectors (tests/golden/crmath_vectors.txt: mpmath at 300
bits, rounded to the nearest double, over the argument ranges the trajectory
uses and their edges) every result must be the correctly rounded one; against
the host C library (whose results the reference's trajectories use) they must
agree on all but a sliver of random arguments, where CUDA's own functions
differ on up to a fifth of them."""
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
