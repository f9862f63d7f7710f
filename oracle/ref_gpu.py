"""The reference's own GPU kernels, run for comparison (test and bench
infrastructure; the product never loads this).

`make -C oracle ref` compiles the reference sources unchanged as CUDA for
sm_103a and device-links them into _ref/ref_gpu.cubin.  This module loads that
cubin through the CUDA driver API (libcuda, the context torch made current) and
runs the reference's GPU path of mainAnalysis (src/simulation.cpp:8-96 with
particle::particle and particle::runSimulation, src/particle.cpp:450-636):
initParticlesGPU once, then runSimulationGPU once per output window,
<<<ceil(N / numPerGPUBlock), numPerGPUBlock>>>, over device arrays laid out as
the reference's (coords = 3 doubles, rngState = 48 bytes, SpectrumAggregator =
2600 bytes; pinned by tests/test_ref_gpu_layout.py against the reference build).
"""
from __future__ import annotations

import ctypes
import math
from pathlib import Path

CUBIN = Path(__file__).resolve().parent / "_ref" / "ref_gpu.cubin"
INIT = ("_Z16initParticlesGPU7optionsP6coordsS1_S1_S1_S1_PdS2_S2_S2_S2_S2_P8rngStatePmS5_S5_PjPiPbPcS9_"
        "P18SpectrumAggregator22floquetDiagonalization")
RUN = ("_Z16runSimulationGPU7optionsP6coordsS1_S1_S1_S1_PdS2_S2_S2_S2_S2_P8rngStatePmS5_S5_PjPiPbPcS9_"
       "P18SpectrumAggregatord")
SIZES = {"options": 440, "coords": 24, "rngState": 48, "SpectrumAggregator": 2600, "floquetDiagonalization": 240}

# the kernels' array arguments after `options`, with their element sizes
ARRAYS = [("S", 24), ("v", 24), ("v_old", 24), ("pos", 24), ("pos_old", 24), ("t", 8), ("t_old", 8), ("tf", 8),
          ("dt", 8), ("next_gas", 8), ("h", 8), ("state", 48), ("n_bounce", 8), ("n_coll", 8), ("n_steps", 8),
          ("partID", 4), ("fail", 4), ("stop", 1), ("coll_type", 1), ("wall_hit", 1), ("specagg", 2600)]


def available() -> bool:
    return CUBIN.exists()


class RefGPU:
    """The loaded cubin and its two kernels (needs a current CUDA context)."""

    def __init__(self):
        import torch
        torch.zeros(1, device="cuda")  # the runtime's primary context, current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), str(CUBIN).encode()), "cuModuleLoad")
        self.init_fn, self.run_fn = ctypes.c_void_p(), ctypes.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(self.init_fn), self.mod, INIT.encode()), "init kernel")
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(self.run_fn), self.mod, RUN.encode()), "run kernel")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: CUDA driver error {rc}")

    def _launch(self, fn, opt_bytes, arrays, last, n, block, stream):
        ob = ctypes.create_string_buffer(bytes(opt_bytes), len(opt_bytes))
        ptrs = [ctypes.c_void_p(a.data_ptr()) for a in arrays]
        params = [ctypes.cast(ob, ctypes.c_void_p)] + [ctypes.cast(ctypes.byref(p), ctypes.c_void_p) for p in ptrs]
        params.append(ctypes.cast(ctypes.byref(last) if not isinstance(last, ctypes.Array) else last, ctypes.c_void_p))
        argv = (ctypes.c_void_p * len(params))(*params)
        grid = (n + block - 1) // block
        self._check(self.cu.cuLaunchKernel(fn, ctypes.c_uint(grid), 1, 1, ctypes.c_uint(block), 1, 1, 0,
                                           ctypes.c_void_p(stream), argv, None), "cuLaunchKernel")

    def run(self, opt, windows: int, device: int = 0):
        """mainAnalysis's GPU path without the file: init, then `windows`
        windows.  opt is an options image (440 bytes, derived as mainAnalysis
        does).  Returns (seconds on the stream, dict of host arrays)."""
        import numpy as np
        import torch
        n = int(opt.numParticles)
        block = int(opt.numPerGPUBlock) or 128
        dev = torch.device("cuda", device)
        arrays = [torch.zeros(max(n, 1) * size, dtype=torch.uint8, device=dev) for _, size in ARRAYS]
        stream = torch.cuda.current_stream(dev)
        fd = ctypes.create_string_buffer(SIZES["floquetDiagonalization"])  # integrator types 0-5 ignore it
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        self._launch(self.init_fn, bytes(opt), arrays, fd, n, block, stream.cuda_stream)
        for w in range(windows):
            self._launch(self.run_fn, bytes(opt), arrays, ctypes.c_double((w + 1.0) * opt.ioutInt), n, block,
                         stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        secs = e0.elapsed_time(e1) / 1e3
        host = {name: a.cpu().numpy() for (name, _), a in zip(ARRAYS, arrays)}
        out = {"t": host["t"].view(np.float64)[:n], "pos": host["pos"].view(np.float64)[:3 * n].reshape(n, 3),
               "v": host["v"].view(np.float64)[:3 * n].reshape(n, 3),
               "S": host["S"].view(np.float64)[:3 * n].reshape(n, 3), "fail": host["fail"].view(np.int32)[:n],
               "n_coll": host["n_coll"].view(np.uint64)[:n], "n_bounce": host["n_bounce"].view(np.uint64)[:n],
               "n_steps": host["n_steps"].view(np.uint64)[:n]}
        del arrays
        return secs, out


def windows_of(opt) -> int:
    """floor((tf - t0) / ioutInt), as mainAnalysis counts its windows."""
    return int(math.floor((opt.tf - opt.t0) / opt.ioutInt))
