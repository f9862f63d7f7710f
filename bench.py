"""Throughput of the spin-tracking hot path on GB300: particle*seconds simulated
per wall second (DOP853, rtol = atol = 1e-12, FP64).

Workload (default): the plain-at-scale configuration -- 1,048,576 particles,
Maxwell-Boltzmann at 4.2 K, cosine-law diffuse walls (0.1), gravity, the full
3x3 linear gradient tensor with entries N(0, 1e-9) T/m (numpy default_rng(0)),
E = (0, 0, 75e5) V/m, B0 = (3e-6, 0, 0) T, output every 0.5 s -- with two
deliberate changes, both recorded in the JSON `config`:
  * gas collisions off: at 4.2 K the reference's free time
    tc = 1.6e-4 m / (k T^8) is 1.44 ps (~7e11 collisions per particle-second),
    which no implementation can integrate;
  * tf = 1 s instead of 100 s (two output windows), so a step takes seconds;
    the metric is a rate, so it is unchanged by the shortening.
A step = one pass of the hot path over the batch: initialise every particle
on the device, then run every output window with the batched persistent
kernel, snapshots written to a device buffer.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU implementation on this
host's cores (the C restatement in oracle/, which reproduces the reference
build bit for bit) on bounded samples of the same workload; beside it, under
"reference_gpu", the reference's own CUDA kernels built unchanged for sm_103a
(when their cubin was built with the reference sources present) on a sample.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "spin-tracking_gb300"))

import numpy as np  # noqa: E402

METRIC = "particle·s simulated/s (DOP853 rtol 1e-12), batched+adjoint vs plain, 1 GB300"
UNIT = "particle*s/s"
WORKLOAD = ("plain-at-scale: 1,048,576 particles, MB 4.2 K, diffuse 0.1, gravity, full G ~ N(0,1e-9) T/m, "
            "E=(0,0,75e5), B0=(3e-6,0,0), DOP853 rtol 1e-12, ioutInt 0.5 s; gas collisions off (tc = 1.44 ps "
            "at 4.2 K is intractable); tf = 1 s")


def workload_fields(n: int, tf: float, first: int = 0) -> dict:
    """The workload's options for particles [first, first + n) of the full run.
    A shard seeds as the reference does (seed + global index) by offsetting
    the seed: (seed + first) + i == seed + (first + i) in 32-bit arithmetic."""
    g = np.random.default_rng(0).normal(0.0, 1e-9, 9)
    return dict(
        numParticles=n, dist=b"M", T=4.2, m=1.20239e-26, gamma=-2.038e8, diffuse=0.1, gas_coll=False, gravity=True,
        L=(0.07, 0.1, 0.4), B0=(3e-6, 0.0, 0.0), E=(0.0, 0.0, 75e5), yi=(0.0, 0.0, 1.0), Gx=tuple(g[0:3]),
        Gy=tuple(g[3:6]), Gz=tuple(g[6:9]), t0=0.0, tf=tf, ioutInt=0.5, rtol=1e-12, atol=1e-12, h=1e-3, hmax=1.0,
        hmin=1e-8, integratorType=0, seed=(0 + first) & 0xFFFFFFFF, maxPosStep=0.1, a=0.0, w=0.0)


def apply_fields(opt, fields: dict):
    for k, v in fields.items():
        if isinstance(v, tuple):
            cur = getattr(opt, k)
            cur.x, cur.y, cur.z = (float(x) for x in v)
        else:
            setattr(opt, k, v)
    return opt


def workload_options(n: int, tf: float, first: int = 0):
    import spintrack as st
    return st.derive(apply_fields(st.default_options(), workload_fields(n, tf, first)))


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        rows = []
        for l in self.lines:
            p = [x.strip() for x in l.split(",")]
            if len(p) < 8:
                continue
            try:
                rows.append((float(p[0]), float(p[1]), p[4:8]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i in range(4) if r[i].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------- dist
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def shard(n_total: int, world: int, rank: int) -> tuple[int, int]:
    """Particles [first, first + n) of rank `rank`: equal shards, the last one
    takes the remainder."""
    per = n_total // world
    first = rank * per
    return first, (per if rank < world - 1 else n_total - first)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU baseline
def cpu_sample_rate(tf: float, target_s: float, first: int = 0):
    """Time the oracle (reference algorithm, C) on a bounded sample of the
    workload with every host core.  Returns (rate, cores, sample text)."""
    sys.path.insert(0, str(REPO / "tests"))
    from _oracle import Oracle
    orc = Oracle()
    cores = os.cpu_count() or 1
    opt = apply_fields(orc.default_options(), workload_fields(1, tf))
    orc.L.or_derive(ctypes.byref(opt))
    # calibrate on a small sample, then size the measured sample to target_s
    n = max(cores * 4, 64)
    secs, _ = orc.run_sample(opt, first, n, threads=cores)
    per_particle = max(secs, 1e-6) / n
    n = int(min(max(n, target_s / per_particle), 1 << 20))
    secs, _ = orc.run_sample(opt, first, n, threads=cores)
    sim = (int((tf - 0.0) / 0.5)) * 0.5
    return n * sim / secs, cores, f"particles [{first}, {first + n}) of the workload, t = 0..{sim:g} s, {secs:.1f} s wall"


def reference_gpu_rate(args):
    """The reference's own CUDA kernels (initParticlesGPU, then runSimulationGPU
    once per window, built unchanged for sm_103a into the oracle's reference
    cubin and launched through the driver API) on a sample of the workload: a
    calibration run of 8,192 particles, then one run sized to about
    --ref-gpu-seconds (one thread per particle: a sample much larger than the
    GPU's 38,912 resident threads, so that the last particles do not decide),
    timed with CUDA events on the launching stream."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no GPU"}
        sys.path.insert(0, str(REPO / "oracle"))
        sys.path.insert(0, str(REPO / "tests"))
        import ref_gpu
        from _oracle import Oracle
        if not ref_gpu.available():
            return {"unavailable": "reference cubin not built (it needs the reference sources at build time)"}
        orc = Oracle()
        kern = ref_gpu.RefGPU()

        def opts(n):
            o = apply_fields(orc.default_options(), workload_fields(n, args.tf))
            orc.L.or_derive(ctypes.byref(o))
            return o
        n = 8192
        secs, _ = kern.run(opts(n), ref_gpu.windows_of(opts(n)))
        n = int(min(max(n, args.ref_gpu_seconds / max(secs, 1e-6) * n), args.particles))
        o = opts(n)
        nw = ref_gpu.windows_of(o)
        secs, out = kern.run(o, nw)
        sim = nw * o.ioutInt
        return {"value": n * sim / secs, "unit": UNIT, "particles": n, "tf": sim, "seconds": secs,
                "block": int(o.numPerGPUBlock), "stopped": int((out["fail"] != 0).sum()),
                "kernels": "the reference's initParticlesGPU + runSimulationGPU per window (src/particle.cpp:450-636), "
                           "one thread per particle, built unchanged for sm_103a"}
    except Exception as e:  # the comparison is informative; the CPU line stands without it
        return {"unavailable": f"{type(e).__name__}: {e}"}


# ---------------------------------------------------------------- adjoint
ADJ_WORKLOAD = ("adjoint: 65,536 particles, MB 4.2 K, specular walls, gravity, gas off, full G ~ N(0,1e-9) T/m, "
                "E=(0,0,75e5), B0=(3e-6,0,0), DOP853 rtol 1e-12, tf = 1 s (shortened from 50 s), gradients of "
                "<Sx> w.r.t. G(9), B0(3), E(3); the whole tape held in HBM (no replay); record and backward "
                "timed after one untimed record + backward")


def adjoint_timing(args, dev):
    import torch
    import spintrack as st
    g = np.random.default_rng(0).normal(0.0, 1e-9, 9)
    n = 65536
    opt = st.derive(st.make_options(numParticles=n, dist="M", T=4.2, diffuse=0.0, gas_coll=False, gravity=True,
                                    Gx=g[0:3], Gy=g[3:6], Gz=g[6:9], E=(0, 0, 75e5), B0=(3e-6, 0, 0), yi=(0, 0, 1),
                                    tf=1.0, ioutInt=0.5, seed=0))
    nw = st.num_windows(opt)
    with st.Particles(opt, device=dev) as p:
        def timed(fn):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            return time.perf_counter() - t0
        p.init_particles()
        p.run_windows(0, nw, st.KERNEL_PERSISTENT)
        p.init_particles()
        t_fwd = timed(lambda: p.run_windows(0, nw, st.KERNEL_PERSISTENT))
        w = torch.zeros(n, 3, dtype=torch.float64, device=f"cuda:{dev}")
        w[:, 0] = 1.0 / n
        out = torch.empty(n, 17, dtype=torch.float64, device=f"cuda:{dev}")
        p.init_particles()
        p.adjoint_record(nw)  # allocates the tape pool
        p.adjoint_backward(w.data_ptr(), out.data_ptr())
        p.init_particles()
        t_rec = timed(lambda: p.adjoint_record(nw))
        t_bwd = timed(lambda: p.adjoint_backward(w.data_ptr(), out.data_ptr()))
        stats = p.adjoint_stats()
        finite = bool(torch.isfinite(out).all().item())
        del w, out
        torch.cuda.synchronize()
    return {"workload": ADJ_WORKLOAD, "forward_batched_s": t_fwd, "record_s": t_rec, "backward_s": t_bwd,
            "backward_over_forward": t_bwd / t_fwd, "record_plus_backward_over_forward": (t_rec + t_bwd) / t_fwd,
            "tape_gb": stats["tape_bytes_used"] / 1e9, "tape_resident": bool(stats["resident"]),
            "replays": stats["replays"], "gradients_finite": finite}


# ---------------------------------------------------------------- configuration workloads
# Opt-in lines (--workload); the default run prints only the headline line.
WORKLOADS = {
    "sweep": "batched parameter sets: 4096 sets x 256 particles (seed_s = 256 s), per set B0 = (U[1,10] uT, 0, 0), "
             "9 gradient entries U[0,1e-8] T/m, E_z = +-75e5 V/m, diffuse U[0,0.5], gas collisions at T = 0.4 K, "
             "sets 0-2047 DOP853 with tf U[0.01,1] s, sets 2048-4095 RK45 with tf U[1e-5,1e-3] s (tf shortened from "
             "U[1,100] s: RK45 at rtol 1e-12 takes ~20M attempts per particle-second), one window per set",
    "adjoint50": "adjoint at full length: 65,536 particles, MB 4.2 K, specular walls, gravity, gas off, "
                 "G ~ N(0,1e-9) T/m, E = (0,0,75e5), B0 = (3e-6,0,0), tf = 50 s, ioutInt 0.5 s; gradients of <Sx>, "
                 "<Sy> and the mean precession phase; the tape (~1.2 TB) exceeds HBM, so the backward replays "
                 "window chunks from state checkpoints",
    "literal-gas": "plain-at-scale as written: gas collisions at T = 4.2 K, whose clock tc = 1.44 ps gives ~7e11 "
                   "collisions per particle-second; 65,536 particles, tf shortened to 2 ns (~1,400 collisions per "
                   "particle), otherwise the headline workload",
    "dressing": "spin dressing: 262,144 particles, a = 5e-6 T, w = 2 pi 1000 rad/s (z pulse), B0 = (3e-6,0,0), "
                "diffuse 0.5, gas collisions at T = 0.4 K, gravity, hmax = 1e-4, tf = 1 s (shortened from 20 s), "
                "ioutInt 0.5 s",
    "adjoint-small": "adjoint, small case for profiles: 65,536 particles (the lanes of the backward as full), MB "
                     "4.2 K, specular walls, gravity, gas off, G ~ N(0,1e-9) T/m, E = (0,0,75e5), B0 = (3e-6,0,0), "
                     "tf = 0.05 s, tape pool 3 GB (the tape, ~0.9 GB, stays resident); gradients of <Sx>, <Sy> and "
                     "the mean precession phase",
    "integrators": "the six integrator types on the headline physics (262,144 particles, MB 4.2 K, diffuse 0.1, "
                   "gravity, full G, E = (0,0,75e5), B0 = (3e-6,0,0), gas off): DOP853 rtol 1e-12 tf 0.05 s, RK45 "
                   "rtol 1e-12 tf 5e-5 s, Magnus CFET8 rtol 1e-12 tf 0.05 s, RK45 with quaternions rtol 1e-10 tf "
                   "0.0125 s, RKF45 rtol 1e-3 tf 0.005 s, RKF45 with quaternions rtol 1e-6 tf 2.5e-4 s (the RKF45 "
                   "pair's error estimates are the whole increment and the last stage's rotation: they accept "
                   "only steps of ~3 us and ~0.1 us, and tighter tolerances fail with h < hmin), one window each",
    "adjoint-magnus": "adjoint of the Magnus CFET8 stepper: 65,536 particles, MB 4.2 K, specular walls, gravity, gas "
                      "off, G ~ N(0,1e-9) T/m, E = (0,0,75e5), B0 = (3e-6,0,0), integratorType 2, rtol 1e-12, "
                      "tf = 1 s, ioutInt 0.5 s; gradients of <Sx>, <Sy> and the mean precession phase",
    "dressing-grid": "dressing sensitivity: 8 x 8 grid a in [1,10] uT, w in 2 pi [500,2000] rad/s as 64 parameter "
                     "sets x 4096 particles in one context, otherwise as 'dressing' with tf = 0.2 s; d<P>/d(a, w) of "
                     "the polarisation P = |<S>| per grid point from one record + one backward pass",
}


def _set_options(n, tf, seed=0, **kw):
    import spintrack as st
    f = workload_fields(n, tf)
    f.update(seed=seed & 0xFFFFFFFF)
    f.update(kw)
    return st.derive(apply_fields(st.default_options(), f))


def sweep_sets():
    r = np.random.default_rng(3)
    sets = []
    for s in range(4096):
        dop = s < 2048
        tf = r.uniform(0.01, 1.0) if dop else r.uniform(1e-5, 1e-3)
        g = r.uniform(0.0, 1e-8, 9)
        sets.append(_set_options(256, tf, seed=s * 256, T=0.4, gas_coll=True, diffuse=r.uniform(0.0, 0.5),
                                 B0=(r.uniform(1e-6, 1e-5), 0.0, 0.0), Gx=tuple(g[0:3]), Gy=tuple(g[3:6]),
                                 Gz=tuple(g[6:9]), E=(0.0, 0.0, 75e5 if r.uniform() < 0.5 else -75e5), ioutInt=tf,
                                 integratorType=0 if dop else 1))
    return sets


def dressing_options(n, tf, a=5e-6, w=2 * np.pi * 1000.0):
    return _set_options(n, tf, T=0.4, gas_coll=True, diffuse=0.5, a=a, w=w, hmax=1e-4,
                        ioutInt=min(0.5, tf))


def _timed_forward(p, nwin, steps, warmup, dev):
    """Device-timed steps (init + all windows) on the engine's stream."""
    import torch
    import spintrack as st
    stream = torch.cuda.ExternalStream(p.stream(), device=dev)

    def step():
        p.init_particles()
        rc = p.run_windows(0, nwin, st.KERNEL_PERSISTENT)
        if rc != 0:
            raise RuntimeError(f"run_windows returned {rc}")
    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / steps, clk.summary()


def run_workload(args):
    import torch
    import spintrack as st
    from spintrack import _capi, workmodel
    from spintrack.adjoint import NUM_THETA
    dev = 0
    torch.cuda.set_device(dev)
    peak = ctypes.c_double()
    _capi.check(_capi.load().st_probe_fp64_peak(dev, ctypes.byref(peak)))
    line = {"workload": args.workload, "description": WORKLOADS[args.workload], "n_gpus": 1, "dtype": "f64",
            "data": "synthetic"}

    def roofline(counters, secs, ext_type=None):
        ach = workmodel.algorithmic_flops(counters, ext_type) / secs / 1e12
        return {"bound": "fp64", "achieved": ach, "peak": peak.value, "unit": "TFLOP/s", "frac": ach / peak.value}

    if args.workload == "integrators":
        names = {0: "DOP853", 1: "RK45", 2: "Magnus CFET8", 3: "RK45 quaternion", 4: "RKF45", 5: "RKF45 quaternion"}
        plan = ((0, 1e-12, 0.05), (1, 1e-12, 5e-5), (2, 1e-12, 0.05), (3, 1e-10, 0.0125), (4, 1e-3, 0.005),
                (5, 1e-6, 2.5e-4))
        per = []
        want = {int(x) for x in args.types.split(",") if x.strip()}
        npt = args.type_particles
        for it, rtol, tf in plan:
            if it not in want:
                continue
            o = _set_options(npt, tf, integratorType=it, rtol=rtol, ioutInt=tf)
            with st.Particles(o, device=dev) as p:
                if args.variant >= 0:
                    p.set_launch_config(args.variant, args.bps)
                secs, clk = _timed_forward(p, 1, args.steps, 1, dev)
                c = p.counters()
                att = c["dop_attempts"] + c["rk45_attempts"] + c["ext_attempts"]
                per.append({"integratorType": it, "name": names[it], "rtol": rtol, "tf": tf,
                            "particles": npt, "value": npt * tf / secs, "ms_per_step": secs * 1e3, "attempts": att,
                            "attempts_per_s": att / secs, "segments": c["segments"],
                            "failed": int(np.count_nonzero(p.output_data()["fail"])),
                            "roofline": roofline(c, secs, it if it >= 2 else None),
                            "launch_config": list(p.launch_config()), "clocks": clk})
        line.update({"metric": "particle*s simulated/s per integrator type", "unit": "particle*s/s",
                     "steps": args.steps, "warmup": 1, "per_type": per})
        return line

    if args.workload in ("sweep", "dressing", "literal-gas"):
        if args.workload == "sweep":
            sets = sweep_sets()
        elif args.workload == "dressing":
            sets = [dressing_options(args.dressing_particles, args.dressing_tf)]
        else:
            sets = [_set_options(65536, 2e-9, gas_coll=True, ioutInt=2e-9)]
        psec = sum(int(o.numParticles) * st.num_windows(o) * o.ioutInt for o in sets)
        nwin = max(st.num_windows(o) for o in sets)
        with st.Particles(sets, device=dev) as p:
            if args.variant >= 0:
                p.set_launch_config(args.variant, args.bps)
            secs, clk = _timed_forward(p, nwin, args.steps, 1, dev)
            c = p.counters()
            line.update({"metric": "particle*s simulated/s", "value": psec / secs, "unit": "particle*s/s",
                         "ms_per_step": secs * 1e3, "steps": args.steps, "warmup": 1, "particle_seconds": psec,
                         "counters": {k: c[k] for k in ("dop_attempts", "rk45_attempts", "segments")},
                         "roofline": roofline(c, secs), "launch_config": list(p.launch_config()), "clocks": clk})
            if args.workload == "sweep":
                half = [sum(int(o.numParticles) * o.tf for o in sets[a:b]) for a, b in ((0, 2048), (2048, 4096))]
                line["particle_seconds_dop853_rk45"] = half
        return line

    tape_bytes = 0
    if args.workload in ("adjoint50", "adjoint-small", "adjoint-magnus"):
        g = np.random.default_rng(0).normal(0.0, 1e-9, 9)
        small = args.workload == "adjoint-small"
        magnus = args.workload == "adjoint-magnus"
        tf = 0.05 if small else (1.0 if magnus else 50.0)
        opt = _set_options(65536, tf, diffuse=0.0, Gx=tuple(g[0:3]), Gy=tuple(g[3:6]), Gz=tuple(g[6:9]),
                           ioutInt=0.05 if small else 0.5, integratorType=2 if magnus else 0)
        sets = [opt]
        tape_bytes = 3_000_000_000 if small else 0
    else:
        av = np.linspace(1e-6, 10e-6, 8)
        wv = 2 * np.pi * np.linspace(500.0, 2000.0, 8)
        sets = [dressing_options(4096, 0.2, a=a, w=w) for a in av for w in wv]
    nwin = max(st.num_windows(o) for o in sets)
    n = sum(int(o.numParticles) for o in sets)
    pulse = args.workload == "dressing-grid"

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0
    with st.Particles(sets, device=dev) as p:
        p.init_particles()
        p.run_windows(0, nwin, st.KERNEL_PERSISTENT)  # tunes the launch configuration
        p.init_particles()
        t_fwd = timed(lambda: p.run_windows(0, nwin, st.KERNEL_PERSISTENT))
        p.init_particles()
        t_rec = timed(lambda: p.adjoint_record(nwin, tape_bytes=tape_bytes))
        stats = p.adjoint_stats()
        S = torch.empty(n, 3, dtype=torch.float64, device=f"cuda:{dev}")
        torch.cuda.synchronize()
        p.gather_spins(S.data_ptr())
        torch.cuda.synchronize()
        out = torch.empty(n, NUM_THETA, dtype=torch.float64, device=f"cuda:{dev}")
        counts = [int(o.numParticles) for o in sets]
        losses = {}
        if pulse:
            w = torch.zeros_like(S)
            for k, part in enumerate(S.split(counts)):
                m = part.mean(0)
                lo = sum(counts[:k])
                w[lo:lo + counts[k]] = (m / m.norm()) / counts[k]
            losses["P"] = w
        else:
            ok = torch.isfinite(S).all(1)
            nv = float(ok.sum().item())
            wx = torch.zeros_like(S)
            wx[ok, 0] = 1.0 / nv
            wy = torch.zeros_like(S)
            wy[ok, 1] = 1.0 / nv
            r2 = S[:, 1] ** 2 + S[:, 2] ** 2
            wp = torch.zeros_like(S)
            wp[ok, 1] = (-S[ok, 2] / r2[ok]) / nv
            wp[ok, 2] = (S[ok, 1] / r2[ok]) / nv
            losses = {"Sx": wx, "Sy": wy, "phase": wp}
        t_bwd = {}
        grads = {}
        for name, wgt in losses.items():
            wgt = wgt.contiguous()
            t_bwd[name] = timed(lambda: p.adjoint_backward(wgt.data_ptr(), out.data_ptr(), pulse))
            per_set = torch.stack([c.sum(0) for c in out.split(counts)])
            grads[name] = per_set.cpu().numpy()
        bstats = p.adjoint_stats()
        t_multi = None
        if len(losses) > 1:  # all losses in one backward: one replay per chunk serves them all
            wall = torch.stack([w.contiguous() for w in losses.values()]).contiguous()
            outm = torch.empty(len(losses), n, NUM_THETA, dtype=torch.float64, device=f"cuda:{dev}")
            t_multi = timed(lambda: p.adjoint_backward_multi(len(losses), wall.data_ptr(), outm.data_ptr(), pulse))
            for k, name in enumerate(losses):
                assert np.array_equal(torch.stack([c.sum(0) for c in outm[k].split(counts)]).cpu().numpy(),
                                      grads[name])
    tb = sum(t_bwd.values()) / len(t_bwd)
    line.update({"metric": "adjoint seconds", "unit": "s", "particles": n, "windows": nwin,
                 "forward_batched_s": t_fwd, "record_s": t_rec, "backward_s": t_bwd,
                 "backward_over_forward": tb / t_fwd, "record_plus_backward_over_forward": (t_rec + tb) / t_fwd,
                 "tape_gb": stats["tape_bytes_used"] / 1e9, "pool_gb": stats["tape_bytes_pool"] / 1e9,
                 "tape_resident": bool(stats["resident"]), "checkpoints": stats["checkpoints"],
                 "replays_per_backward": bstats["replays"], "groups_per_backward": bstats["groups"],
                 "tail_from_checkpoint": stats["tail_from"], "record_launches": stats["record_launches"],
                 "backward_all_losses_one_call_s": t_multi})
    if pulse:
        g = grads["P"]
        line["dP_da_grid"] = g[:, 15].reshape(8, 8).tolist()
        line["dP_dw_grid"] = g[:, 16].reshape(8, 8).tolist()
        line["gradients_finite"] = bool(np.isfinite(g[:, 15:17]).all())
    else:
        line["gradients"] = {k: v[0].tolist() for k, v in grads.items()}
        line["gradients_finite"] = all(bool(np.isfinite(v).all()) for v in grads.values())
    return line


# ---------------------------------------------------------------- main
def workload_config(args, world):
    """The `config` object of both arms' lines: the workload and its sizes."""
    sim = int(args.tf / 0.5) * 0.5
    return {"workload": WORKLOAD, "particles": args.particles, "tf": sim, "windows": int(args.tf / 0.5),
            "l2": "inputs larger than L2: per-particle state 178 MB + snapshot blocks, rewritten each step",
            "parallelism": f"particle shards x{world}"}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    rates = []
    sample = ""
    cores = os.cpu_count() or 1
    for i in range(args.warmup + args.steps):
        r, cores, sample = cpu_sample_rate(args.tf, args.ref_step_seconds, first=i * 4096)
        if i >= args.warmup:
            rates.append(r)
    v = statistics.mean(rates)
    # the same workload keys as the repo arm's line; the CPU times a bounded
    # sample of it each step (particles are independent and seeded by their
    # global index, so the rate of a sample is the rate of the workload)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, 1),
            "sample_per_step": sample,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.skip_reference_gpu:
        line["reference_gpu"] = reference_gpu_rate(args)
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, world, rank, local):
    import torch
    import spintrack as st
    from spintrack import _capi, workmodel

    lib = _capi.load()
    dev = local
    torch.cuda.set_device(dev)
    n_total = args.particles
    first, n = shard(n_total, world, rank)
    opt = workload_options(n, args.tf, first)
    nwin = st.num_windows(opt)
    sim = nwin * opt.ioutInt

    peak = ctypes.c_double()
    _capi.check(lib.st_probe_fp64_peak(dev, ctypes.byref(peak)))

    p = st.Particles(opt, device=dev)
    if args.variant >= 0:
        p.set_launch_config(args.variant, args.bps)
    stream = torch.cuda.ExternalStream(p.stream(), device=dev)
    snap = torch.empty(p.snapshot_bytes() * nwin, dtype=torch.uint8, device=f"cuda:{dev}")
    kernel = st.KERNEL_PLAIN if args.kernel == "plain" else st.KERNEL_PERSISTENT

    def step(k=kernel):
        p.init_particles()
        rc = p.run_windows(0, nwin, k, snap.data_ptr())
        if rc != 0:
            raise RuntimeError(f"run_windows returned {rc}")

    for _ in range(args.warmup):
        step()
    counters = p.counters()
    lcfg = p.launch_config()
    lcfg_name = st.variant_name(lcfg[0]) if lcfg[0] >= 0 else None

    # ---- timed region: K steps, CUDA events on the launching stream
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    k_events = []
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        launches = 0
        for _ in range(args.steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            p.init_particles()
            launches += 1
            a.record(stream)
            rc = p.run_windows(0, nwin, kernel, snap.data_ptr())
            b.record(stream)
            if rc != 0:
                raise RuntimeError(f"run_windows returned {rc}")
            launches += p.counters()["kernel_launches"]
            k_events.append((a, b))
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    elapsed = ev0.elapsed_time(ev1) * 1e-3
    elapsed = max_over_ranks(world, elapsed)
    kernel_s = statistics.mean(a.elapsed_time(b) * 1e-3 for a, b in k_events)
    counters = p.counters()
    ms_per_step = elapsed / args.steps * 1e3
    value = n_total * sim * args.steps / elapsed

    flops = workmodel.algorithmic_flops(counters)
    achieved = flops / kernel_s * 1e-12
    roof = {"bound": "fp64", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
            "frac": achieved / peak.value if peak.value else None, "traffic": None,
            "peak_source": "measured: DFMA issue-rate probe in this run (no FP64 entry in MEASURED_PEAKS.json; "
                           "nominal GB300 FP64 1.25 TFLOP/s)",
            "work_per_launch": {"dop_attempts": counters["dop_attempts"], "segments": counters["segments"],
                                "flops": flops, "kernel_ms": kernel_s * 1e3}}
    # DRAM bytes of one launch, from an ncu capture of dram__bytes_read.sum + dram__bytes_write.sum
    # (one pass) of this kernel on this workload at its full size, 1,048,576 particles and two
    # windows: 279.85 MB read (the state, once) + 453.40 MB written (the state and a snapshot block
    # at each window end), 699 B per particle per two windows; other sizes scale by particles and
    # windows (every particle's state and snapshot cross DRAM once per window end).
    roof["traffic"] = 733.3e6 * (n / 1048576.0) * (nwin / 2.0)
    roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum of this kernel on the full "
                              "workload (1,048,576 particles, 2 windows: 733.3 MB), scaled to this launch")

    # ---- plain one-thread-per-particle kernel on the same workload (1 step)
    plain = None
    if not args.skip_plain and kernel != st.KERNEL_PLAIN:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step(st.KERNEL_PLAIN)
        torch.cuda.synchronize()
        tp = time.perf_counter() - t0
        tp = max_over_ranks(world, tp)
        plain = {"value": n_total * sim / tp, "ms_per_step": tp * 1e3, "speedup_of_batched": (n_total * sim / tp)
                 and value / (n_total * sim / tp)}

    # ---- end to end through the public API with host buffers
    host = torch.empty(snap.numel(), dtype=torch.uint8, pin_memory=True)
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        p.set_params(opt)            # H2D: the parameter table from host memory
        p.init_particles()
        p.run_windows(0, nwin, kernel, snap.data_ptr())
        with torch.cuda.stream(stream):
            host.copy_(snap, non_blocking=True)   # D2H: every window's snapshot block
        stream.synchronize()
    te = (time.perf_counter() - t0) / e2e_steps
    te = max_over_ranks(world, te)
    e2e = {"value": n_total * sim / te, "unit": UNIT, "h2d_bytes_per_step": p.param_table_bytes() * world,
           "d2h_bytes_per_step": int(snap.numel()) * world, "ms_per_step": te * 1e3}

    # ---- discrete adjoint on the adjoint workload shape (65,536 particles,
    # specular walls, tf = 1 s): record pass + backward vs a forward pass
    adjoint = None
    if not args.skip_adjoint and rank == 0:
        adjoint = adjoint_timing(args, dev)

    cpu = None
    if rank == 0 and not args.skip_cpu:
        rate, cores, sample = cpu_sample_rate(args.tf, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}

    clocks = clk.summary()
    # release the torch buffers that ran on the engine's stream before the
    # stream and context go away
    torch.cuda.synchronize()
    del host, snap, stream
    import gc
    gc.collect()
    torch.cuda.synchronize()
    p.close()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config(args, world),
                "kernel": args.kernel,
                "launch_config": {"variant": lcfg[0], "name": lcfg_name, "blocks_per_sm": lcfg[1]},
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "plain_kernel": plain, "adjoint": adjoint,
                "gpu_launches": launches, "clocks": clocks}
        print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--particles", type=int, default=1 << 20)
    ap.add_argument("--tf", type=float, default=1.0)
    ap.add_argument("--kernel", choices=["persistent", "plain"], default="persistent")
    ap.add_argument("--variant", type=int, default=-1, help="persistent-kernel variant (-1: autotune)")
    ap.add_argument("--bps", type=int, default=0, help="resident blocks per SM with --variant")
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-adjoint", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--ref-gpu-seconds", type=float, default=30.0,
                    help="reference arm: target duration of the reference GPU kernels' sample")
    ap.add_argument("--skip-reference-gpu", action="store_true",
                    help="reference arm: leave out the timing of the reference's own GPU kernels")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=None,
                    help="print the line of one additional configuration instead of the headline line")
    ap.add_argument("--dressing-particles", type=int, default=262144,
                    help="particles of the 'dressing' workload (smaller for profiles)")
    ap.add_argument("--dressing-tf", type=float, default=1.0, help="simulated time of the 'dressing' workload")
    ap.add_argument("--types", type=str, default="0,1,2,3,4,5",
                    help="integrator types of the 'integrators' workload (comma-separated)")
    ap.add_argument("--type-particles", type=int, default=262144,
                    help="particles per integrator type in the 'integrators' workload")
    args = ap.parse_args()
    if args.workload:
        print(json.dumps(run_workload(args)), flush=True)
        return 0
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_ours(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
