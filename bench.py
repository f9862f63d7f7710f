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
build bit for bit) on bounded samples of the same workload.
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


# ---------------------------------------------------------------- main
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
    sim = int(args.tf / 0.5) * 0.5
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "particles_per_step": "bounded sample", "tf": sim},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
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
    per = n_total // world
    first = rank * per
    n = per if rank < world - 1 else n_total - first
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
    tr = REPO / "profiles" / "traffic.json"
    if tr.exists():
        try:
            t = json.loads(tr.read_text())
            roof["traffic"] = t.get("bytes_per_launch_scaled")
        except Exception:
            pass

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
                "config": {"workload": WORKLOAD, "particles": n_total, "tf": sim, "windows": nwin,
                           "kernel": args.kernel, "launch_config": {"variant": lcfg[0], "blocks_per_sm": lcfg[1]},
                           "l2": "inputs larger than L2: per-particle state 178 MB + snapshot blocks, rewritten each step",
                           "parallelism": f"particle shards x{world}"},
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
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_ours(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
