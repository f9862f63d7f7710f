"""Differentiable spin tracking: a torch.autograd.Function over the engine's
discrete adjoint (st_adjoint_record / st_adjoint_backward).

theta has one row per parameter set, ST_NUM_THETA = 17 columns:
    Gx(3), Gy(3), Gz(3)  rows of the linear gradient tensor (B_i = pos . G_i), T/m
    B0(3)                holding field, T
    E(3)                 electric field, V/m
    a, w                 pulse amplitude (T) and angular frequency (rad/s)
The forward returns the final spins (N x 3, float64, on the engine's device);
gradients are exact for the accepted step sequence of that forward pass (the
adaptive step choice is held fixed), with the DOP853 or the Magnus CFET8
stepper (integratorType 0 or 2, one per engine).
"""
from __future__ import annotations

import math

import torch

from ._capi import Options, Vec3

NUM_THETA = 17
THETA_NAMES = ("Gx.x", "Gx.y", "Gx.z", "Gy.x", "Gy.y", "Gy.z", "Gz.x", "Gz.y", "Gz.z",
               "B0.x", "B0.y", "B0.z", "E.x", "E.y", "E.z", "a", "w")
_VEC = (("Gx", 0), ("Gy", 3), ("Gz", 6), ("B0", 9), ("E", 12))


def theta_of(opt: Options) -> list[float]:
    th = [0.0] * NUM_THETA
    for name, off in _VEC:
        v = getattr(opt, name)
        th[off:off + 3] = [v.x, v.y, v.z]
    th[15], th[16] = opt.a, opt.w
    return th


def with_theta(opt: Options, theta) -> Options:
    o = Options.from_buffer_copy(bytes(opt))
    t = [float(x) for x in theta]
    for name, off in _VEC:
        setattr(o, name, Vec3(*t[off:off + 3]))
    o.a, o.w = t[15], t[16]
    return o


class TrackSpins(torch.autograd.Function):
    """S_final = track(theta); backward runs the engine's discrete adjoint."""

    @staticmethod
    def forward(ctx, theta, engine, base_sets, w_end, pulse):
        th = theta.detach().to("cpu", torch.float64)
        sets = [with_theta(o, th[k]) for k, o in enumerate(base_sets)]
        engine.set_params(sets)
        engine.init_particles()
        engine.adjoint_record(w_end)
        dev = torch.device("cuda", engine.device)
        S = torch.empty(engine.n, 3, dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        engine.gather_spins(S.data_ptr())
        ctx.engine = engine
        ctx.pulse = bool(pulse)
        ctx.counts = [int(o.numParticles) for o in base_sets]
        ctx.theta_device = theta.device
        return S

    @staticmethod
    def backward(ctx, gS):
        eng = ctx.engine
        dev = torch.device("cuda", eng.device)
        g = torch.nan_to_num(gS.detach().to(dev, torch.float64).contiguous(), nan=0.0)
        out = torch.empty(eng.n, NUM_THETA, dtype=torch.float64, device=dev)
        torch.cuda.synchronize(dev)
        eng.adjoint_backward(g.data_ptr(), out.data_ptr(), ctx.pulse)
        per_set = torch.stack([c.sum(0) for c in out.split(ctx.counts)]) if ctx.counts else out.new_zeros(0, NUM_THETA)
        return per_set.to(ctx.theta_device), None, None, None, None


def track_spins(theta: torch.Tensor, engine, base_sets, w_end: int, pulse: bool = False) -> torch.Tensor:
    """Final spins of every particle as a differentiable function of theta (nsets x 17)."""
    return TrackSpins.apply(theta, engine, list(base_sets), int(w_end), pulse)


def precession_phase(S: torch.Tensor) -> torch.Tensor:
    """Precession angle about x, atan2(Sz, Sy), as the reference's analysis
    scripts define it (scripts/nedmSim.py, benchmarks notebooks)."""
    return torch.atan2(S[:, 2], S[:, 1])
