"""torch.autograd bridge to the discrete adjoint, for checks against finite
differences and an FP64 reference adjoint: ``TetTraces.apply(eps_r, sim,
nsteps, nsnap)`` runs the recorded forward of a TetFemSimulation (or
TetFemBatch) and returns its receiver traces as a tensor; ``backward`` hands
dJ/dtraces to ``ems_tetfem_backward`` and returns dJ/deps_r.  The tensors
are host FP64 tensors: the simulation holds its own device state."""
import numpy as np
import torch


class TetTraces(torch.autograd.Function):
    @staticmethod
    def forward(ctx, eps_r, sim, nsteps, nsnap):
        sim.set_material(eps_r.detach().cpu().numpy().astype(np.float64))
        sim.set_checkpoints(nsnap)
        sim.reset()
        sim.run(nsteps)
        ctx.sim = sim
        return torch.from_numpy(sim.traces().copy())

    @staticmethod
    def backward(ctx, grad_traces):
        g = ctx.sim.backward(grad_traces.detach().cpu().numpy().astype(np.float64))
        return torch.from_numpy(g), None, None, None
