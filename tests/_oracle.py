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


NW = 17  # Goertzel frequencies of integratorType 6


class Spec(ctypes.Structure):
    """or_spec: one particle's noise-spectrum aggregator."""
    _fields_ = [("s1", Vec3 * NW), ("s2", Vec3 * NW), ("imag", Vec3 * NW), ("n_samples", ctypes.c_int64)]


class Particles(ctypes.Structure):
    _fields_ = [("n", c_int)] + [(k, POINTER(Vec3)) for k in ("S", "v", "v_old", "pos", "pos_old")] + \
               [(k, POINTER(c_double)) for k in ("t", "t_old", "h", "next_gas")] + \
               [("rng", POINTER(Rng)), ("fail", POINTER(c_int))] + \
               [(k, POINTER(c_uint64)) for k in ("n_bounce", "n_coll", "n_steps")] + \
               [("stop", POINTER(ctypes.c_bool)), ("coll_type", POINTER(c_char)), ("wall_hit", POINTER(c_char)),
                ("spec", POINTER(Spec))]


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
            "or_floquet_frequencies": (None, [P(Options), P(c_double), P(c_double)]),
            "or_set_math_mode": (None, [c_int]),
            "or_set_math_pick": (None, [c_void_p]),
            "or_set_math_audit": (None, [c_void_p, c_void_p, c_void_p, c_void_p, c_int]),
            "or_math_eval": (None, [c_int, c_int, c_void_p, c_void_p, ctypes.c_int64, c_int]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        self.L = L
        assert L.or_options_size() == 440

    # elementary functions of the trajectory ------------------------------
    MATH_LIBM, MATH_CR, MATH_AUDIT, MATH_PICK = 0, 1, 2, 3
    FN = {"log": 0, "sin": 1, "cos": 2, "acos": 3}
    FN_NAMES = {v: k for k, v in FN.items()}

    def math_eval(self, fn: str, x, correctly_rounded: bool, threads: int = 0):
        """fn(x) elementwise: the host C library, or correctly rounded
        (binary128 evaluation rounded once)."""
        import numpy as np
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        self.L.or_math_eval(self.FN[fn], 1 if correctly_rounded else 0, x.ctypes.data, y.ctypes.data, x.size,
                            threads)
        return y

    def set_math_mode(self, mode: int) -> None:
        self.L.or_set_math_mode(mode)

    def run_sample_audited(self, opt: Options, first: int, count: int, threads: int = 0, mode: int = 2,
                           snapshots: bool = False, pick=None):
        """run_sample with the trajectory's elementary functions in `mode`
        (MATH_AUDIT: the host library; MATH_CR: correctly rounded; MATH_PICK:
        correctly rounded but for the pick[i]-th call of particle i whose
        host result differs), each call audited against the other result.
        Returns (seconds, arrays, audit) where audit holds per particle the
        number of calls whose host result was not correctly rounded and, for
        the first, the particle time at the start of its segment, the function
        and the argument.  With snapshots=True the arrays are a list over the
        snapshots t0, t0 + ioutInt, ...; the math mode is restored to the host
        library on return."""
        import numpy as np
        cnt = np.zeros(count, np.int64)
        t1 = np.full(count, np.inf)
        fn = np.full(count, -1, np.int32)
        arg = np.full(count, np.nan)
        pk = np.ascontiguousarray(pick if pick is not None else np.full(count, -1), dtype=np.int64)
        self.L.or_set_math_pick(pk.ctypes.data)
        self.L.or_set_math_mode(mode)
        self.L.or_set_math_audit(cnt.ctypes.data, t1.ctypes.data, fn.ctypes.data, arg.ctypes.data, count)
        p = self.alloc(count)
        try:
            if snapshots:
                nwin = int(np.floor((opt.tf - opt.t0) / opt.ioutInt))
                t0 = __import__("time").perf_counter()
                self.L.or_init(ctypes.byref(opt), ctypes.byref(p), first)
                out = [self.arrays(p)]
                for w in range(nwin):
                    self.L.or_run_until(ctypes.byref(opt), ctypes.byref(p), (w + 1.0) * opt.ioutInt, threads)
                    out.append(self.arrays(p))
                secs = __import__("time").perf_counter() - t0
            else:
                secs = self.L.or_run_sample(ctypes.byref(opt), first, count, threads, ctypes.byref(p))
                out = self.arrays(p)
        finally:
            self.free(p)
            self.L.or_set_math_audit(None, None, None, None, 0)
            self.L.or_set_math_pick(None)
            self.L.or_set_math_mode(self.MATH_LIBM)
        return secs, out, {"count": cnt, "first_t": t1, "first_fn": fn, "first_arg": arg}

    # integratorType 6: noise spectrum -----------------------------------
    def floquet_frequencies(self, opt: Options):
        """floquet_diagonalize's 17 Goertzel frequencies and dt."""
        import numpy as np
        f = (c_double * NW)()
        dt = c_double()
        self.L.or_floquet_frequencies(ctypes.byref(opt), f, ctypes.byref(dt))
        return np.array(f[:]), dt.value

    def run_spectrum(self, opt: Options, first: int, count: int, threads: int = 0, math_mode: int = 0):
        """Particles [first, first + count) of a type-6 run through every
        window; returns (arrays, spectrum) where spectrum holds each particle's
        aggregator at the end of the last window: s1, s2, imag [count, 17, 3]
        and n_samples [count].  math_mode: the trajectory's elementary
        functions (MATH_LIBM, the reference's, or MATH_CR)."""
        import numpy as np
        p = self.alloc(count)
        self.L.or_set_math_mode(math_mode)
        try:
            self.L.or_run_sample(ctypes.byref(opt), first, count, threads, ctypes.byref(p))
            out = self.arrays(p)
            spec = {"s1": np.zeros((count, NW, 3)), "s2": np.zeros((count, NW, 3)), "imag": np.zeros((count, NW, 3)),
                    "n_samples": np.zeros(count, np.int64)}
            if p.spec:
                for i in range(count):
                    g = p.spec[i]
                    for k in range(NW):
                        for name in ("s1", "s2", "imag"):
                            v = getattr(g, name)[k]
                            spec[name][i, k] = (v.x, v.y, v.z)
                    spec["n_samples"][i] = g.n_samples
        finally:
            self.L.or_set_math_mode(self.MATH_LIBM)
            self.free(p)
        return out, spec

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
