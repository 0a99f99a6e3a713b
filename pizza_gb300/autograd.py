"""PyTorch gradient path: the time-averaged kinetic energy of a pizza run as a
differentiable function of the initial temperature perturbation and Ra.

``kinetic_energy(temp0, ra, ensemble, n_steps, n_window)`` returns, per
instance, J = mean over the last ``n_window`` states of
us2_3D + up2_3D + uz2_3D (pizza's e_kin_3D columns, src/outputs.f90:553-570);
``nusselt_top`` the mean of NuTop (the heat file's first Nusselt number).
Its backward runs the hand-written discrete adjoint of the CNAB2 step
(``pz_adjoint_backward``) with checkpointing and recomputation.  The time-step
sequence is the one the Courant controller picks in the forward sweep (or the
one given as ``dt_sched``) and is held fixed in the gradient.

Gradients follow PyTorch's complex convention: for real J and complex z,
``z.grad`` is g with dJ = Re(sum(conj(g) dz)).
"""
from __future__ import annotations

import numpy as np
import torch

from . import Ensemble


class KineticEnergy(torch.autograd.Function):
    """J(temp0, ra) for every instance of an Ensemble: the time-averaged
    kinetic energy ('ekin3d') or outer-boundary Nusselt number ('nutop').

    temp0: complex128 tensor (n_instances, n_m_max, n_r_max) (all instances of
    one shape) -- the temp argument of pz_set_state; ra: float64 tensor
    (n_instances,)."""

    @staticmethod
    def forward(ctx, temp0, ra, ens: Ensemble, n_steps: int, n_window: int, checkpoint_every: int, dt_sched,
                objective: str = "ekin3d"):
        temps = temp0.detach().cpu().numpy()
        ras = ra.detach().cpu().numpy().astype(np.float64)
        if temps.shape[0] != len(ens) or ras.shape != (len(ens),):
            raise ValueError("temp0 and ra need one entry per instance")
        for i in range(len(ens)):
            ens.set_ra(i, float(ras[i]))
        ens.set_state_all([temps[i] for i in range(len(ens))])
        J, dt_used = ens.adjoint_forward(n_steps, n_window, checkpoint_every, dt_sched, objective)
        ctx.ens = ens
        ctx.device = temp0.device
        ctx.dt_used = dt_used
        return torch.as_tensor(J, dtype=torch.float64, device=temp0.device)

    @staticmethod
    def backward(ctx, grad_J):
        g, dra = ctx.ens.adjoint_backward()
        gJ = grad_J.detach().to("cpu", torch.float64).numpy()
        gT = torch.as_tensor(np.stack(g) * gJ[:, None, None], device=ctx.device)
        gR = torch.as_tensor(dra * gJ, device=ctx.device)
        return gT, gR, None, None, None, None, None, None


def kinetic_energy(temp0, ra, ens: Ensemble, n_steps: int, n_window: int, checkpoint_every: int = 0,
                   dt_sched=None):
    """Differentiable J (float64 tensor, one value per instance)."""
    return KineticEnergy.apply(temp0, ra, ens, int(n_steps), int(n_window), int(checkpoint_every), dt_sched)


def nusselt_top(temp0, ra, ens: Ensemble, n_steps: int, n_window: int, checkpoint_every: int = 0,
                dt_sched=None):
    """Differentiable mean of NuTop (src/outputs.f90:742-746) over the last
    n_window states, one value per instance."""
    return KineticEnergy.apply(temp0, ra, ens, int(n_steps), int(n_window), int(checkpoint_every), dt_sched,
                               "nutop")
