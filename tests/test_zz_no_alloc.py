"""The allocation-free entry point (st_run_noalloc) against the allocating one.

st_run_noalloc exists for callers that cannot call cudaMalloc when they run
the tracker (a host whose memory pool owns the GPU, or a hot path that must
not synchronise the device through cudaMalloc/cudaFree): they hand in one
device buffer for the particle state and the library uses only a scratch array
compiled into it.  This test allocates that buffer itself (the entry point does
not), runs the same parameter sets through st_run_noalloc twice in a row and
through st_create_batch + st_init + st_run_windows, and requires the same
results: counts exact, spin within 1e-9, trajectory within 1e-7 (the
tolerances of the golden parity tests).  The file is collected last so that a
run stopping at the first failure has run every other test first.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from conftest import GOLDEN
import spintrack as st
from spintrack import _capi

pytestmark = pytest.mark.gpu


def _sets(names=("m04_gas", "c1_precess")):
    return [st.derive(st.parse_params(GOLDEN / f"{c}.params")) for c in names]


def _reference(sets, nwin):
    with st.Particles(sets) as p:
        p.init_particles()
        p.run_windows(0, nwin, st.KERNEL_PERSISTENT)
        return p.output_data()


def _fields_from_buffer(buf, n):
    """The first 14 arrays of the caller buffer (256-byte aligned each)."""
    raw = buf.cpu().numpy()
    off = 0
    out = {}
    sizes = [("t", 8, np.float64), ("px", 8, np.float64), ("py", 8, np.float64), ("pz", 8, np.float64),
             ("vx", 8, np.float64), ("vy", 8, np.float64), ("vz", 8, np.float64), ("Sx", 8, np.float64),
             ("Sy", 8, np.float64), ("Sz", 8, np.float64), ("fail", 4, np.int32), ("n_coll", 8, np.uint64),
             ("n_bounce", 8, np.uint64), ("n_steps", 8, np.uint64)]
    for name, sz, dt in sizes:
        out[name] = raw[off:off + sz * n].view(dt).copy()
        off += (sz * max(n, 1) + 255) // 256 * 256
    return {"t": out["t"], "pos": np.stack([out["px"], out["py"], out["pz"]], 1),
            "v": np.stack([out["vx"], out["vy"], out["vz"]], 1), "S": np.stack([out["Sx"], out["Sy"], out["Sz"]], 1),
            "fail": out["fail"], "n_coll": out["n_coll"], "n_bounce": out["n_bounce"], "n_steps": out["n_steps"]}


def _close(got, ref):
    for f in ("fail", "n_coll", "n_bounce", "n_steps"):
        np.testing.assert_array_equal(got[f], ref[f], err_msg=f)
    for f, tol in (("t", 1e-7), ("pos", 1e-7), ("v", 1e-7), ("S", 1e-9)):
        a, b = got[f], ref[f]
        assert np.array_equal(np.isnan(a), np.isnan(b)), f
        m = ~np.isnan(b)
        assert np.all(np.abs(a[m] - b[m]) <= tol * np.maximum(1.0, np.abs(b[m]))), f


@pytest.mark.parametrize("names", [("m04_gas", "c1_precess"), ("magnus", "rkf45q", "rk45")],
                         ids=["dop853", "types-2-5"])
def test_noalloc_matches_allocating_path_twice(gpu, names):
    import torch
    lib = _capi.load()
    sets = _sets(names)
    nwin = min(st.num_windows(s) for s in sets)
    n = sum(int(s.numParticles) for s in sets)
    arr = (st.Options * len(sets))(*sets)
    need = ctypes.c_size_t(0)
    assert lib.st_run_noalloc(arr, len(sets), None, ctypes.byref(need), nwin, None) == 0
    assert need.value > 0
    ref = _reference(sets, nwin)
    buf = torch.empty(need.value, dtype=torch.uint8, device=gpu)   # the caller's allocation
    assert buf.data_ptr() % 256 == 0
    stream = torch.cuda.current_stream(gpu)
    for call in range(2):  # the scratch keeps the previous call's contents: both calls must agree
        sz = ctypes.c_size_t(need.value)
        rc = lib.st_run_noalloc(arr, len(sets), ctypes.c_void_p(buf.data_ptr()), ctypes.byref(sz), nwin,
                                ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, lib.st_last_error()
        _close(_fields_from_buffer(buf, n), ref)


def test_noalloc_rejects_beyond_limits(gpu):
    lib = _capi.load()
    s = _sets()[0]
    nine = (st.Options * 9)(*([s] * 9))
    sz = ctypes.c_size_t(0)
    assert lib.st_run_noalloc(nine, 9, None, ctypes.byref(sz), 1, None) == _capi.ST_ERR_ARG
    assert b"8 parameter sets" in lib.st_last_error()
    one = (st.Options * 1)(s)
    assert lib.st_run_noalloc(one, 1, None, ctypes.byref(sz), 1, None) == 0
    small = ctypes.c_size_t(sz.value - 1)
    assert lib.st_run_noalloc(one, 1, ctypes.c_void_p(256), ctypes.byref(small), 1, None) == _capi.ST_ERR_ARG
