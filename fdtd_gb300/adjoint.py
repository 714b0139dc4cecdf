"""Probe-energy figure of merit as a torch.autograd.Function over the C ABI adjoint.

    J(eps_r) = sum_m dt * Ez(probe)^2 over `steps` steps of a scenario whose design region takes the
    per-cell permittivity eps_r. forward runs fdtd_adjoint_forward (checkpoints every K steps, or
    the design-region E of every step for K = 0); backward runs fdtd_adjoint_backward, the discrete
    adjoint of the FP32 update accumulated in FP64, and scales it by the incoming gradient.

The reference has no gradient; this replaces finite-difference or gradient-free (its commented-out
differential-evolution optimiser, fdtdrav.h:2758-2986) design loops.
"""
from __future__ import annotations

from typing import Optional, Sequence

import numpy as np
import torch

from . import scenario as S
from .solver import Simulation


class ProbeEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps_r: torch.Tensor, sc: "S.Scenario", box: Sequence[int], probe: Sequence[int], steps: int,
                checkpoint_every: int = 64, material_index: Optional[np.ndarray] = None):
        sim = Simulation.from_scenario(sc, material_index=material_index, probe_capacity=max(steps, 1))
        try:
            sim.set_design_region(box, eps_r.detach().to("cpu", torch.float32).numpy())
            J = sim.adjoint_forward(steps, probe, checkpoint_every)
        except Exception:
            sim.close()
            raise
        ctx.sim = sim
        ctx.eps_meta = (eps_r.dtype, eps_r.device)
        return torch.tensor(J, dtype=torch.float64, device=eps_r.device)

    @staticmethod
    def backward(ctx, grad_J: torch.Tensor):
        sim = ctx.sim
        try:
            g = sim.adjoint_backward()
        finally:
            sim.close()
            ctx.sim = None
        dtype, device = ctx.eps_meta
        grad = torch.from_numpy(g).to(device=device) * grad_J.to(torch.float64)
        return grad.to(dtype), None, None, None, None, None, None


def probe_energy(eps_r: torch.Tensor, sc: "S.Scenario", box: Sequence[int], probe: Sequence[int], steps: int,
                 checkpoint_every: int = 64, material_index: Optional[np.ndarray] = None) -> torch.Tensor:
    """Differentiable J(eps_r); eps_r shaped (box[5]-box[2], box[4]-box[1], box[3]-box[0])."""
    return ProbeEnergy.apply(eps_r, sc, tuple(box), tuple(probe), int(steps), int(checkpoint_every), material_index)
