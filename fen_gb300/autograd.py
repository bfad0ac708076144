"""torch.autograd.Function over the discrete adjoint (a thin ctypes harness).

``Rollout.apply(u0, v0, solver, nsteps, dt)`` runs nsteps FP64 steps of a 2D periodic
context from the initial velocity (u0, v0) (FEN host layout, CPU float64 tensors) and returns
the final (u, v); its backward calls the library's checkpointed adjoint.  p and dv_o start
from the values already in the solver.
"""
import numpy as np
import torch

from . import U, V


class Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u0, v0, solver, nsteps, dt, every=50):
        solver.set_field(U, u0.detach().cpu().numpy())
        solver.set_field(V, v0.detach().cpu().numpy())
        solver.update_ghost_nodes(U)
        solver.update_ghost_nodes(V)
        solver.set_dt_o(dt)
        solver.adjoint_setup(nsteps, every)
        solver.adjoint_forward(dt)
        ctx.solver = solver
        uT = torch.from_numpy(solver.get_field(U))
        vT = torch.from_numpy(solver.get_field(V))
        return uT, vT

    @staticmethod
    def backward(ctx, gu, gv):
        g_u, g_v, _ = ctx.solver.adjoint_backward(gu.detach().cpu().numpy().astype(np.float64),
                                                  gv.detach().cpu().numpy().astype(np.float64))
        return torch.from_numpy(g_u), torch.from_numpy(g_v), None, None, None, None
