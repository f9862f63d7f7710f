"""ctypes binding of include/spintrack.h (the engine's C ABI).

Loading fails loudly when libspintrack.so has not been built: there is no
CPU fallback for any computation.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_bool, c_char, c_char_p, c_double, c_int, c_int32, c_int64, c_size_t, c_uint, c_uint8, c_uint64, c_void_p
from pathlib import Path

from . import build as _build


class Vec3(ctypes.Structure):
    _fields_ = [("x", c_double), ("y", c_double), ("z", c_double)]


class Options(ctypes.Structure):
    """st_options: field-for-field the reference's `struct options`
    (include/options.h:10-61), 440 bytes, also the format-'A' header."""

    _fields_ = [
        ("B0", Vec3), ("E", Vec3), ("L", Vec3), ("yi", Vec3), ("Gx", Vec3), ("Gy", Vec3), ("Gz", Vec3),
        ("m", c_double), ("t0", c_double), ("tf", c_double), ("rtol", c_double), ("atol", c_double),
        ("beta", c_double), ("uround", c_double), ("safe", c_double), ("fac1", c_double), ("fac2", c_double),
        ("hmax", c_double), ("hmin", c_double), ("h", c_double), ("T", c_double), ("sqrtKT_m", c_double),
        ("tc", c_double), ("gamma", c_double), ("V", c_double), ("a", c_double), ("w", c_double),
        ("swapStepSize", c_double), ("maxPosStep", c_double), ("ioutInt", c_double), ("diffuse", c_double),
        ("nmax", c_uint), ("seed", c_uint), ("integratorType", c_int), ("numParticles", c_int),
        ("numPerGPUBlock", c_int), ("iout", c_int), ("dist", c_char), ("gas_coll", c_bool), ("gravity", c_bool),
        ("fixedStepSize", c_bool), ("keepStepSize", c_bool), ("noiseAmplitudes", Vec3), ("noiseFrequencies", Vec3),
    ]


assert ctypes.sizeof(Options) == 440


class StateView(ctypes.Structure):
    _fields_ = [("t", POINTER(c_double)), ("pos", POINTER(Vec3)), ("v", POINTER(Vec3)), ("S", POINTER(Vec3)),
                ("fail", POINTER(c_int32)), ("n_coll", POINTER(c_uint64)), ("n_bounce", POINTER(c_uint64)),
                ("n_steps", POINTER(c_uint64))]


class DeviceSoA(ctypes.Structure):
    _fields_ = [("n_total", c_int64)] + [(k, c_void_p) for k in (
        "t", "pos_x", "pos_y", "pos_z", "v_x", "v_y", "v_z", "S_x", "S_y", "S_z", "h", "next_gas",
        "fail", "n_coll", "n_bounce", "n_steps", "stop")]


class LaunchConfig(ctypes.Structure):
    _fields_ = [("block_threads", c_int), ("blocks_per_sm", c_int), ("variant", c_int)]


class AdjointStats(ctypes.Structure):
    """st_adjoint_stats."""
    _fields_ = [("tape_bytes_used", c_uint64), ("tape_bytes_pool", c_uint64), ("resident", ctypes.c_int32),
                ("checkpoints", ctypes.c_int32), ("windows_per_checkpoint", ctypes.c_int32),
                ("replays", ctypes.c_int32), ("groups", ctypes.c_int32), ("tail_from", ctypes.c_int32),
                ("record_launches", ctypes.c_int32), ("pad", ctypes.c_int32)]


class Ensemble(ctypes.Structure):
    """st_ensemble."""
    _fields_ = [("t", c_double), ("n_valid", c_int64), ("n_phase", c_int64), ("mean_S", c_double * 3),
                ("polarisation", c_double), ("phase_mean", c_double), ("phase_std", c_double),
                ("phase_stderr", c_double), ("phase_expected", c_double), ("freq_shift", c_double),
                ("freq_shift_err", c_double), ("phase_unwrapped_mean", c_double),
                ("phase_unwrapped_std", c_double), ("freq_shift_unwrapped", c_double)]


class Counters(ctypes.Structure):
    _fields_ = [("dop_attempts", c_uint64), ("rk45_attempts", c_uint64), ("segments", c_uint64),
                ("kernel_launches", c_uint64), ("graph_launches", c_uint64), ("graph_captures", c_uint64),
                ("ext_attempts", c_uint64)]


ST_OK = 0
ST_ERR_ARG = -1
ST_ERR_CUDA = -2
ST_ERR_UNSUPPORTED = -3
ST_ERR_IO = -4
ST_ERR_STATE = -5
ST_ERR_DEADLINE = -6
ST_ERR_NOMEM = -7
KERNEL_PLAIN = 0
KERNEL_PERSISTENT = 1

_SIGS = {
    "st_version": (c_int, []),
    "st_last_error": (c_char_p, []),
    "st_options_size": (c_size_t, []),
    "st_options_default": (None, [POINTER(Options)]),
    "st_parse_line": (c_int, [POINTER(Options), c_char_p]),
    "st_parse_params": (c_int, [c_char_p, POINTER(Options)]),
    "st_derive": (None, [POINTER(Options)]),
    "st_num_windows": (c_int, [POINTER(Options)]),
    "st_create": (c_int, [POINTER(Options), c_int, POINTER(c_void_p)]),
    "st_create_batch": (c_int, [POINTER(Options), c_int, c_int, POINTER(c_void_p)]),
    "st_destroy": (None, [c_void_p]),
    "st_init": (c_int, [c_void_p]),
    "st_run_until": (c_int, [c_void_p, c_double]),
    "st_run_windows": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p]),
    "st_snapshot_bytes": (c_size_t, [c_void_p]),
    "st_snapshot_field_offset": (c_size_t, [c_void_p, c_int]),
    "st_read_state": (c_int, [c_void_p, POINTER(StateView)]),
    "st_device_state": (c_int, [c_void_p, POINTER(DeviceSoA)]),
    "st_gather_spins": (c_int, [c_void_p, c_void_p]),
    "st_synchronize": (c_int, [c_void_p]),
    "st_get_stream": (c_void_p, [c_void_p]),
    "st_set_params": (c_int, [c_void_p, POINTER(Options), c_int]),
    "st_param_table_bytes": (c_size_t, [c_void_p]),
    "st_set_launch_config": (c_int, [c_void_p, POINTER(LaunchConfig)]),
    "st_get_launch_config": (c_int, [c_void_p, POINTER(LaunchConfig)]),
    "st_set_deadline": (c_int, [c_void_p, c_double]),
    "st_launch_variant_count": (c_int, []),
    "st_launch_variant_name": (c_char_p, [c_int]),
    "st_get_counters": (c_int, [c_void_p, POINTER(Counters)]),
    "st_main_analysis": (c_int, [POINTER(Options), c_char_p, c_int, c_int, POINTER(c_double)]),
    "st_crmath_eval": (c_int, [c_int, c_void_p, c_void_p, ctypes.c_int64]),
    "st_probe_fp64_peak": (c_int, [c_int, POINTER(c_double)]),
    "st_adjoint_record": (c_int, [c_void_p, c_int, c_size_t, c_int]),
    "st_adjoint_get_stats": (c_int, [c_void_p, POINTER(AdjointStats)]),
    "st_floquet_frequencies": (c_int, [POINTER(Options), POINTER(c_double), POINTER(c_double)]),
    "st_spectrum_state": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "st_covariance_spectrum": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "st_ensemble_stats": (c_int, [c_void_p, c_void_p, c_int, POINTER(Ensemble)]),
    "st_gather_phase": (c_int, [c_void_p, c_void_p]),
    "st_adjoint_backward": (c_int, [c_void_p, c_void_p, c_void_p, c_int]),
    "st_adjoint_backward_multi": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int]),
    "st_run_noalloc": (c_int, [POINTER(Options), c_int, c_void_p, POINTER(c_size_t), c_int, c_void_p]),
    "st_write_header": (c_int, [c_void_p, POINTER(Options)]),
    "st_write_snapshot": (c_int, [c_void_p, c_int, POINTER(StateView)]),
}

_lib = None


class SpinTrackError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"spintrack error {code}: {msg}")
        self.code = code


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libspintrack.so (optionally building it first)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build the CUDA engine first (python -c 'import __graft_entry__ as g; g.build()')")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> int:
    if rc < 0:
        raise SpinTrackError(rc, (load().st_last_error() or b"").decode(errors="replace"))
    return rc
