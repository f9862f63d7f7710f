"""spintrack — Python front-end of the GB300 spin-tracking engine.

Mirrors the reference's host interface for the hot path:
  optionParser / parseLine  -> parse_params / parse_line
  class particle            -> Particles (init_particles, run_simulation,
                               output_data), plus the batched window driver
  mainAnalysis              -> main_analysis (writes output format 'A')
Every computation runs in libspintrack.so on the GPU (no CPU fallback).
"""
from __future__ import annotations

import ctypes
import math
from pathlib import Path
from typing import Iterable

import numpy as np

from . import build
from ._capi import (KERNEL_PERSISTENT, KERNEL_PLAIN, ST_ERR_DEADLINE, AdjointStats, Counters, Ensemble, DeviceSoA, LaunchConfig, Options,
                    SpinTrackError, StateView, Vec3, check, load)
from .formats import read_format_a, snapshot_dtype

__all__ = [
    "Options", "Vec3", "Particles", "SpinTrackError", "default_options", "parse_params", "parse_line",
    "derive", "num_windows", "make_options", "main_analysis", "read_format_a", "KERNEL_PLAIN",
    "KERNEL_PERSISTENT", "SNAP_FIELDS",
]

SNAP_FIELDS = ("t", "pos_x", "pos_y", "pos_z", "v_x", "v_y", "v_z", "S_x", "S_y", "S_z", "fail", "n_coll",
               "n_bounce", "n_steps", "turns")
_SNAP_DTYPES = (np.float64,) * 10 + (np.int32, np.uint64, np.uint64, np.uint64, np.int32)


def default_options() -> Options:
    """options{} defaults (include/options.h:10-61)."""
    o = Options()
    load().st_options_default(ctypes.byref(o))
    return o


def parse_line(opt: Options, line: str) -> int:
    """parseLine (src/optionsParser.cpp:40-175): 0 applied, 1 unrecognised key."""
    return check(load().st_parse_line(ctypes.byref(opt), line.encode()))


def parse_params(path: str | Path) -> Options:
    """optionParser (src/optionsParser.cpp:177-197)."""
    o = Options()
    rc = load().st_parse_params(str(path).encode(), ctypes.byref(o))
    if rc not in (0, -4):  # a missing file keeps the defaults, as the reference does
        check(rc)
    return o


def derive(opt: Options) -> Options:
    """tc and sqrtKT_m as mainAnalysis derives them (src/simulation.cpp:9-11)."""
    load().st_derive(ctypes.byref(opt))
    return opt


def num_windows(opt: Options) -> int:
    return load().st_num_windows(ctypes.byref(opt))


def make_options(**kw) -> Options:
    """Defaults overridden by keyword values; vectors as 3-sequences, dist as 'C'/'M'."""
    o = default_options()
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(f"unknown option {k}")
        cur = getattr(o, k)
        if isinstance(cur, Vec3):
            setattr(o, k, Vec3(*map(float, v)))
        elif k == "dist":
            o.dist = v.encode() if isinstance(v, str) else v
        else:
            setattr(o, k, v)
    return o


class Particles:
    """The engine object: the reference's `class particle`
    (include/particle.h:87-314), for one or several parameter sets."""

    def __init__(self, opt: Options | Iterable[Options], device: int = 0, derive_params: bool = False):
        lib = load()
        sets = [opt] if isinstance(opt, Options) else list(opt)
        if derive_params:
            sets = [derive(Options.from_buffer_copy(bytes(s))) for s in sets]
        arr = (Options * len(sets))(*sets)
        self._sets = sets
        self._ctx = ctypes.c_void_p()
        check(lib.st_create_batch(arr, len(sets), device, ctypes.byref(self._ctx)))
        self.n = sum(int(s.numParticles) for s in sets)
        self.device = device

    # -- reference interface -------------------------------------------
    def init_particles(self) -> None:
        """initParticles (include/particle.h:241-252)."""
        check(load().st_init(self._ctx))

    def run_simulation(self, next_t: float) -> None:
        """runSimulation(nextTOut) (src/particle.cpp:865-876): plain kernel."""
        check(load().st_run_until(self._ctx, float(next_t)))

    def output_data(self) -> dict:
        """outputData (src/particle.cpp:852-862): the snapshot fields as numpy arrays."""
        n = self.n
        d = {"t": np.empty(n), "pos": np.empty((n, 3)), "v": np.empty((n, 3)), "S": np.empty((n, 3)),
             "fail": np.empty(n, np.int32), "n_coll": np.empty(n, np.uint64), "n_bounce": np.empty(n, np.uint64),
             "n_steps": np.empty(n, np.uint64)}
        if n == 0:
            return d
        P = lambda a, t: a.ctypes.data_as(ctypes.POINTER(t))  # noqa: E731
        view = StateView(P(d["t"], ctypes.c_double), P(d["pos"], Vec3), P(d["v"], Vec3), P(d["S"], Vec3),
                         P(d["fail"], ctypes.c_int32), P(d["n_coll"], ctypes.c_uint64),
                         P(d["n_bounce"], ctypes.c_uint64), P(d["n_steps"], ctypes.c_uint64))
        check(load().st_read_state(self._ctx, ctypes.byref(view)))
        return d

    # -- window driver ---------------------------------------------------
    def run_windows(self, w_begin: int, w_end: int, kernel: int = KERNEL_PERSISTENT, snap_ptr: int = 0) -> int:
        """Advance windows [w_begin, w_end); snapshot blocks to device pointer snap_ptr (0 = none).
        Returns 0, or ST_ERR_DEADLINE when the device time budget ran out."""
        rc = load().st_run_windows(self._ctx, int(kernel), int(w_begin), int(w_end), ctypes.c_void_p(snap_ptr or None))
        if rc == ST_ERR_DEADLINE:
            return rc
        return check(rc)

    def snapshot_bytes(self) -> int:
        return int(load().st_snapshot_bytes(self._ctx))

    def snapshot_offsets(self) -> list[int]:
        return [int(load().st_snapshot_field_offset(self._ctx, k)) for k in range(len(SNAP_FIELDS))]

    def device_state(self) -> DeviceSoA:
        d = DeviceSoA()
        check(load().st_device_state(self._ctx, ctypes.byref(d)))
        return d

    def set_launch_config(self, variant: int = -1, blocks_per_sm: int = 0) -> None:
        cfg = LaunchConfig(0, int(blocks_per_sm), int(variant))
        check(load().st_set_launch_config(self._ctx, ctypes.byref(cfg)))

    def launch_config(self) -> tuple[int, int]:
        cfg = LaunchConfig()
        check(load().st_get_launch_config(self._ctx, ctypes.byref(cfg)))
        return cfg.variant, cfg.blocks_per_sm

    def set_deadline(self, seconds: float) -> None:
        check(load().st_set_deadline(self._ctx, float(seconds)))

    def spectrum_state(self) -> dict:
        """integratorType 6: every particle's noise-spectrum aggregator after the
        last window (SpectrumAggregator, include/floquet.h:76-95): s1, s2,
        imag [n, 17, 3] and n_samples [n]."""
        n = self.n
        out = {k: np.zeros((n, 17, 3)) for k in ("s1", "s2", "imag")}
        out["n_samples"] = np.zeros(n, np.int64)
        if n:
            check(load().st_spectrum_state(self._ctx, out["s1"].ctypes.data, out["s2"].ctypes.data,
                                           out["imag"].ctypes.data, out["n_samples"].ctypes.data))
        return out

    def covariance_spectrum(self, set_index: int = 0):
        """integratorType 6: the set's covariance spectrum summed over its
        particles, complex [17, 3, 3], and the samples it holds."""
        v = np.zeros(17 * 18)
        ns = np.zeros(1, np.int64)
        check(load().st_covariance_spectrum(self._ctx, int(set_index), v.ctypes.data, ns.ctypes.data))
        v = v.reshape(17, 3, 3, 2)
        return v[..., 0] + 1j * v[..., 1], int(ns[0])

    def counters(self) -> dict:
        c = Counters()
        check(load().st_get_counters(self._ctx, ctypes.byref(c)))
        return {k: int(getattr(c, k)) for k, _ in Counters._fields_}

    def gather_spins(self, dst_ptr: int) -> None:
        """Copy the spins into a dense device array (3 doubles per particle) at dst_ptr."""
        check(load().st_gather_spins(self._ctx, ctypes.c_void_p(dst_ptr)))

    def adjoint_record(self, w_end: int, tape_bytes: int = 0, windows_per_checkpoint: int = 0) -> None:
        """Forward pass writing the adjoint's tape (needs a fresh init_particles).

        tape_bytes: device pool for the tape (0: up to 45% of free memory);
        windows_per_checkpoint: state checkpoints for replays when the tape
        does not fit (0: automatic)."""
        check(load().st_adjoint_record(self._ctx, int(w_end), int(tape_bytes), int(windows_per_checkpoint)))

    def gather_phase(self, dst_ptr: int) -> None:
        """Unwrapped precession phase atan2(Sz, Sy) + 2 pi turns of every particle into a
        dense device array (one double per particle) at dst_ptr."""
        check(load().st_gather_phase(self._ctx, ctypes.c_void_p(dst_ptr)))

    def ensemble(self, set_index: int = 0, snap_ptr: int = 0) -> dict:
        """Mean spin, polarisation, aligned/clipped precession phase and frequency
        shift of one parameter set (st_ensemble_stats), from the current state or
        from the device snapshot block at snap_ptr."""
        e = Ensemble()
        check(load().st_ensemble_stats(self._ctx, ctypes.c_void_p(snap_ptr or None), int(set_index), ctypes.byref(e)))
        d = {k: getattr(e, k) for k, _ in Ensemble._fields_}
        d["mean_S"] = tuple(e.mean_S)
        return d

    def adjoint_stats(self) -> dict:
        """Tape size, pool size, and the replays the last backward needed."""
        s = AdjointStats()
        check(load().st_adjoint_get_stats(self._ctx, ctypes.byref(s)))
        return {k: int(getattr(s, k)) for k, _ in AdjointStats._fields_ if k != "pad"}

    def adjoint_backward_multi(self, nloss: int, dLdS_ptr: int, grad_ptr: int, pulse: bool = False) -> None:
        """nloss blocks of dL/dS (device, 3 doubles per particle each) -> nloss blocks of dL/dtheta
        (device, 17 doubles per particle each); one replay of the run serves all of them."""
        check(load().st_adjoint_backward_multi(self._ctx, int(nloss), ctypes.c_void_p(dLdS_ptr),
                                               ctypes.c_void_p(grad_ptr), 1 if pulse else 0))

    def adjoint_backward(self, dLdS_ptr: int, grad_ptr: int, pulse: bool = False) -> None:
        """dL/dS (device, 3 doubles per particle) -> dL/dtheta per particle (device, 17 doubles)."""
        check(load().st_adjoint_backward(self._ctx, ctypes.c_void_p(dLdS_ptr), ctypes.c_void_p(grad_ptr),
                                         1 if pulse else 0))

    def stream(self) -> int:
        """The context's cudaStream_t as an integer handle."""
        return int(load().st_get_stream(self._ctx) or 0)

    def set_params(self, opt: Options | Iterable[Options]) -> None:
        """Re-upload every set's parameters (same particle counts); call init_particles next."""
        sets = [opt] if isinstance(opt, Options) else list(opt)
        arr = (Options * len(sets))(*sets)
        check(load().st_set_params(self._ctx, arr, len(sets)))
        self._sets = sets

    def param_table_bytes(self) -> int:
        return int(load().st_param_table_bytes(self._ctx))

    def synchronize(self) -> None:
        check(load().st_synchronize(self._ctx))

    def close(self) -> None:
        if self._ctx:
            load().st_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def unpack_snapshots(buf: np.ndarray, n: int, offsets: list[int], block_bytes: int, count: int) -> dict:
    """Split `count` snapshot blocks (raw bytes, host) into per-field arrays [count, n]."""
    out = {}
    raw = buf.view(np.uint8)
    for k, (name, dt) in enumerate(zip(SNAP_FIELDS, _SNAP_DTYPES)):
        sz = np.dtype(dt).itemsize
        arr = np.empty((count, n), dtype=dt)
        for s in range(count):
            base = s * block_bytes + offsets[k]
            arr[s] = raw[base:base + sz * n].view(dt)
        out[name] = arr
    return out


def main_analysis(opt: Options, out_path: str | Path, kernel: int = KERNEL_PERSISTENT, device: int = 0) -> float:
    """mainAnalysis (src/simulation.cpp:8-96): run and write format 'A'.
    Returns the wall seconds of the window loop (excluding file writes)."""
    secs = ctypes.c_double()
    check(load().st_main_analysis(ctypes.byref(opt), str(out_path).encode(), device, int(kernel), ctypes.byref(secs)))
    return secs.value


def variant_name(variant: int) -> str:
    """Name of a persistent-kernel launch variant (st_launch_variant_name)."""
    return load().st_launch_variant_name(int(variant)).decode()


def floquet_frequencies(opt):
    """floquet_diagonalize (src/integrator.cpp:824-867): the 17 Goertzel
    frequencies of opt's dressing field and the Goertzel step dt."""
    f = (ctypes.c_double * 17)()
    dt = ctypes.c_double()
    check(load().st_floquet_frequencies(ctypes.byref(opt), f, ctypes.byref(dt)))
    return np.array(f[:]), dt.value
