"""ctypes access to the ORACLE (oracle/spin_oracle.c) for tests and the bench's
CPU-baseline leg.  Test infrastructure: the product never imports this."""
from __future__ import annotations

import ctypes
import subprocess
from ctypes import POINTER, c_char, c_double, c_int, c_uint64, c_void_p
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent
LIB = REPO / "oracle" / "_build" / "liboracle.so"


def _options_cls():
    import sys
    sys.path.insert(0, str(REPO / "spin-tracking_gb300"))
    from spintrack._capi import Options, Vec3  # same 440-byte layout as or_options
    return Options, Vec3


Options, Vec3 = _options_cls()


class Rng(ctypes.Structure):
    _fields_ = [("x", c_uint64), ("y", c_uint64), ("z", c_uint64), ("w", c_uint64), ("spare", c_double),
                ("has_spare", ctypes.c_bool)]


class Particles(ctypes.Structure):
    _fields_ = [("n", c_int)] + [(k, POINTER(Vec3)) for k in ("S", "v", "v_old", "pos", "pos_old")] + \
               [(k, POINTER(c_double)) for k in ("t", "t_old", "h", "next_gas")] + \
               [("rng", POINTER(Rng)), ("fail", POINTER(c_int))] + \
               [(k, POINTER(c_uint64)) for k in ("n_bounce", "n_coll", "n_steps")] + \
               [("stop", POINTER(ctypes.c_bool)), ("coll_type", POINTER(c_char)), ("wall_hit", POINTER(c_char))]


class Counters(ctypes.Structure):
    _fields_ = [("dop_attempts", c_uint64), ("rk45_attempts", c_uint64), ("segments", c_uint64),
                ("ext_attempts", c_uint64)]


def build() -> None:
    r = subprocess.run(["make", "-C", str(REPO / "oracle"), "port"], capture_output=True, text=True)
    if r.returncode:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")


class Oracle:
    def __init__(self):
        if not LIB.exists():
            build()
        L = ctypes.CDLL(str(LIB))
        P = POINTER
        sig = {
            "or_options_size": (ctypes.c_size_t, []),
            "or_options_default": (None, [P(Options)]),
            "or_parse_line": (c_int, [P(Options), ctypes.c_char_p]),
            "or_parse_file": (c_int, [ctypes.c_char_p, P(Options)]),
            "or_derive": (None, [P(Options)]),
            "or_rng_seed": (None, [P(Rng), ctypes.c_uint, ctypes.c_uint]),
            "or_xoshiro": (c_uint64, [P(Rng)]),
            "or_uniform": (c_double, [P(Rng)]),
            "or_normal": (c_double, [P(Rng), c_double, c_double]),
            "or_particles_alloc": (c_int, [P(Particles), c_int]),
            "or_particles_free": (None, [P(Particles)]),
            "or_init": (None, [P(Options), P(Particles), c_int]),
            "or_run_until": (None, [P(Options), P(Particles), c_double, c_int]),
            "or_integrate_dop": (c_int, [P(Options), c_double, c_double, P(Vec3), P(Vec3), P(Vec3), P(c_double)]),
            "or_integrate_rk45": (c_int, [P(Options), c_double, c_double, P(Vec3), P(Vec3), P(Vec3), P(c_double)]),
            "or_integrate_ext": (c_int, [P(Options), c_double, c_double, P(Vec3), P(Vec3), P(Vec3), P(c_double)]),
            "or_interpolate": (None, [P(Options), c_double, c_double, P(Vec3), P(Vec3), P(Vec3), P(Vec3)]),
            "or_event": (c_int, [P(Options), P(Particles), c_int, c_double]),
            "or_main_analysis": (c_int, [P(Options), ctypes.c_char_p, c_int, P(c_double)]),
            "or_run_sample": (c_double, [P(Options), c_int, c_int, c_int, P(Particles)]),
            "or_set_counters": (None, [c_void_p]),
            "or_set_step_log": (None, [c_void_p, ctypes.c_int64, c_int]),
            "or_step_log_count": (ctypes.c_int64, []),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        self.L = L
        assert L.or_options_size() == 440

    # options -------------------------------------------------------------
    def default_options(self) -> Options:
        o = Options()
        self.L.or_options_default(ctypes.byref(o))
        return o

    def parse_file(self, path, derive: bool = True) -> Options:
        o = Options()
        self.L.or_parse_file(str(path).encode(), ctypes.byref(o))
        if derive:
            self.L.or_derive(ctypes.byref(o))
        return o

    def parse_line(self, opt: Options, line: str) -> int:
        return self.L.or_parse_line(ctypes.byref(opt), line.encode())

    # runs ----------------------------------------------------------------
    def main_analysis(self, opt: Options, out: Path, threads: int = 0) -> float:
        secs = c_double()
        rc = self.L.or_main_analysis(ctypes.byref(opt), str(out).encode(), threads, ctypes.byref(secs))
        if rc:
            raise RuntimeError(f"or_main_analysis failed: {rc}")
        return secs.value

    def alloc(self, n: int) -> Particles:
        p = Particles()
        if self.L.or_particles_alloc(ctypes.byref(p), n):
            raise MemoryError
        return p

    def free(self, p: Particles) -> None:
        self.L.or_particles_free(ctypes.byref(p))

    def run_sample(self, opt: Options, first: int, count: int, threads: int = 0):
        """Particles [first, first+count) of opt's run through every window.
        Returns (seconds, dict of numpy arrays)."""
        import numpy as np
        p = self.alloc(count)
        try:
            secs = self.L.or_run_sample(ctypes.byref(opt), first, count, threads, ctypes.byref(p))
            out = self.arrays(p)
        finally:
            self.free(p)
        return secs, out

    def arrays(self, p: Particles) -> dict:
        import numpy as np
        n = p.n
        v3 = lambda ptr: np.ctypeslib.as_array(ctypes.cast(ptr, POINTER(c_double)), shape=(n * 3,)).reshape(n, 3).copy()  # noqa: E731
        sc = lambda ptr, t: np.ctypeslib.as_array(ctypes.cast(ptr, POINTER(t)), shape=(n,)).copy()  # noqa: E731
        if n == 0:
            return {}
        return {"t": sc(p.t, c_double), "pos": v3(p.pos), "v": v3(p.v), "S": v3(p.S), "fail": sc(p.fail, c_int),
                "n_coll": sc(p.n_coll, c_uint64), "n_bounce": sc(p.n_bounce, c_uint64),
                "n_steps": sc(p.n_steps, c_uint64), "h": sc(p.h, c_double), "next_gas": sc(p.next_gas, c_double)}
