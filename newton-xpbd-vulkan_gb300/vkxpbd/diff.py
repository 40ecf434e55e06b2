"""Differentiable XPBD rollouts for PyTorch.

`Rollout` is a torch.autograd.Function over the GPU solver's hand-written
adjoint (xpbd_rollout / xpbd_rollout_backward): its forward steps the scene
for a number of frames with checkpoints, its backward replays the checkpointed
segments and runs the adjoint of every substep. Inputs that take gradients:
initial positions and velocities, inverse masses, soft_contact_mu (the plane's
friction is the mean of it and shape_material_mu), particle_mu and
soft_contact_restitution.

    sim = DiffSim(config, radii, dt=1/60, substeps=10, frames=60, checkpoint_frames=2)
    x_final = sim(x0, v0, inv_mass, mu, particle_mu, restitution)
    loss = ((x_final.mean(0) - target) ** 2).sum(); loss.backward()

A DiffSim keeps the last rollout for its backward, so call backward before the
next forward.
"""
from __future__ import annotations

import numpy as np
import torch

from . import SolverConfig, XpbdSolver


def _np32(t):
    return np.ascontiguousarray(t.detach().to("cpu", torch.float32).numpy())


class Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, inv_mass, soft_contact_mu, particle_mu, restitution, sim):
        sim.config.soft_contact_mu = float(soft_contact_mu)
        sim.config.particle_mu = float(particle_mu)
        sim.config.soft_contact_restitution = float(restitution)
        sim.solver.update_config(sim.config)
        sim.solver.set_particles(_np32(x0), _np32(v0), _np32(inv_mass), sim.radii, sim.flags)
        sim.solver.rollout(sim.dt, sim.substeps, sim.frames, 1, sim.checkpoint_frames)
        ctx.sim = sim
        ctx.dev = x0.device
        return torch.from_numpy(sim.solver.get_positions()).to(x0.device)

    @staticmethod
    def backward(ctx, grad_x):
        g = ctx.sim.solver.rollout_backward(_np32(grad_x))
        dev = ctx.dev

        def t(a):
            return torch.as_tensor(a, dtype=torch.float32, device=dev)

        return (t(g["x0"]), t(g["v0"]), t(g["inv_mass"]), t(g["soft_contact_mu"]), t(g["particle_mu"]),
                t(g["soft_contact_restitution"]), None)


class DiffSim:
    """A solver set up for differentiable rollouts of n particles (plane + particle contacts)."""

    def __init__(self, config: SolverConfig, radii, flags=None, dt=1.0 / 60.0, substeps=10, frames=60,
                 checkpoint_frames=2):
        self.config = config
        self.radii = np.ascontiguousarray(radii, np.float32)
        n = self.radii.shape[0]
        self.flags = np.ones(n, np.int32) if flags is None else np.ascontiguousarray(flags, np.int32)
        self.dt, self.substeps, self.frames, self.checkpoint_frames = dt, substeps, frames, checkpoint_frames
        self.solver = XpbdSolver()
        self.solver.init(config, n)
        self.solver.finalize_meshes()

    def __call__(self, x0, v0, inv_mass, soft_contact_mu, particle_mu, restitution):
        def s(v):
            return v if torch.is_tensor(v) else torch.tensor(float(v))

        return Rollout.apply(x0, v0, inv_mass, s(soft_contact_mu), s(particle_mu), s(restitution), self)
