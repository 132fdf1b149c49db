"""Gradient of the output pulse energy through the GPU adjoint, as a
``torch.autograd.Function``.

``pulse_energy(sim, alpha, seed_amp, chirp, ...)`` runs the RK4/diffraction
run on the handle ``sim`` (FP64 or mixed precision) with the taper profile ``alpha`` at the
control points ``taper_z``, the initial field ``seed_amp * seed`` and the
energy chirp ``chirp``, and returns the pulse energy as a 0-d float64 tensor.
Its backward pass is the hand-written adjoint of the interpolate-push-deposit-
diffract step (``pf_adjoint_backward``, checkpoints every
``checkpoint_every`` steps), not an autograd trace.  The backward pass must
follow its forward pass on the same handle (the checkpoints live there).
"""
from __future__ import annotations

import numpy as np
import torch


class PulseEnergy(torch.autograd.Function):
    @staticmethod
    def forward(ctx, alpha, seed_amp, chirp, sim, taper_z, seed, nsteps, isteps4diff, h,
                checkpoint_every, qdiffraction):
        a = alpha.detach().cpu().numpy().astype(np.float64)
        sim.set_taper_profile(np.asarray(taper_z, dtype=np.float64), a)
        e = sim.adjoint_forward(nsteps, isteps4diff, qdiffraction, h, checkpoint_every, seed[0],
                                seed[1], float(seed_amp), float(chirp))
        ctx.sim = sim
        ctx.ntaper = len(a)
        ctx.device = alpha.device
        return torch.tensor(e, dtype=torch.float64, device=alpha.device)

    @staticmethod
    def backward(ctx, grad_e):
        g, gs, gc = ctx.sim.adjoint_backward(ctx.ntaper, float(grad_e))
        dev = ctx.device
        return (torch.as_tensor(g, dtype=torch.float64, device=dev),
                torch.tensor(gs, dtype=torch.float64, device=dev),
                torch.tensor(gc, dtype=torch.float64, device=dev),
                None, None, None, None, None, None, None, None)


def pulse_energy(sim, alpha, seed_amp, chirp, taper_z, seed, nsteps, isteps4diff, h,
                 checkpoint_every=64, qdiffraction=True):
    """Differentiable pulse energy (see the module docstring)."""
    alpha = torch.as_tensor(alpha, dtype=torch.float64)
    seed_amp = torch.as_tensor(seed_amp, dtype=torch.float64)
    chirp = torch.as_tensor(chirp, dtype=torch.float64)
    return PulseEnergy.apply(alpha, seed_amp, chirp, sim, taper_z, seed, nsteps, isteps4diff, h,
                             checkpoint_every, qdiffraction)
