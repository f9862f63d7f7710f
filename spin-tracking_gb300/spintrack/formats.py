"""Output format 'A' (the reference's BinaryLogger, src/logger.cpp:14-38).

File = the 440-byte options image (include/options.h:10-61), then for every
snapshot (t0 and each window end) eight blocks over the N particles:
t f64, pos {x,y,z} f64, v, S, failureState i32, n_coll u64, n_bounce u64,
n_steps u64 (108 N bytes per snapshot).

The reader is pure numpy and derives the header layout from the same ctypes
structure as the C ABI, not from the reference's stale Python reader.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from ._capi import Options

HEADER_BYTES = 440
# bytes 389..391 are struct padding after keepStepSize; their content is
# unspecified in the reference's files and zero in ours
PAD_SLICE = slice(Options.keepStepSize.offset + 1, Options.noiseAmplitudes.offset)
HEADER_DTYPE = np.dtype(Options)


def snapshot_dtype(n: int) -> np.dtype:
    return np.dtype([
        ("t", "<f8", (n,)), ("pos", "<f8", (n, 3)), ("v", "<f8", (n, 3)), ("S", "<f8", (n, 3)),
        ("fail", "<i4", (n,)), ("n_coll", "<u8", (n,)), ("n_bounce", "<u8", (n,)), ("n_steps", "<u8", (n,)),
    ])


def options_from_bytes(b: bytes) -> Options:
    assert len(b) >= HEADER_BYTES
    return Options.from_buffer_copy(b[:HEADER_BYTES])


def read_format_a(path: str | Path):
    """Return (Options, snapshots) where snapshots is a structured array of
    shape [nsnap] with fields t[N], pos[N,3], v[N,3], S[N,3], fail[N],
    n_coll[N], n_bounce[N], n_steps[N]."""
    raw = Path(path).read_bytes()
    opt = options_from_bytes(raw)
    n = int(opt.numParticles)
    dt = snapshot_dtype(n)
    body = raw[HEADER_BYTES:]
    if n == 0:
        return opt, np.zeros(0, dtype=dt)
    if len(body) % dt.itemsize:
        raise ValueError(f"{path}: body of {len(body)} bytes is not a whole number of {dt.itemsize}-byte snapshots")
    return opt, np.frombuffer(body, dtype=dt)


def header_equal(a: bytes, b: bytes) -> bool:
    """Header images equal up to the unspecified padding bytes."""
    x = bytearray(a[:HEADER_BYTES])
    y = bytearray(b[:HEADER_BYTES])
    x[PAD_SLICE] = bytes(PAD_SLICE.stop - PAD_SLICE.start)
    y[PAD_SLICE] = bytes(PAD_SLICE.stop - PAD_SLICE.start)
    return x == y


def options_to_dict(opt: Options) -> dict:
    out = {}
    for name, typ in Options._fields_:
        v = getattr(opt, name)
        if isinstance(v, ctypes.Structure):
            v = (v.x, v.y, v.z)
        elif isinstance(v, bytes):
            v = v.decode("latin-1")
        out[name] = v
    return out
