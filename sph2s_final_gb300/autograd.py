"""torch.autograd bridge for the differentiable rollout (gradient harness only;
the solver itself does not link torch).

    loss = DensityFieldLoss.apply(v0, mu, solver, dt, steps, checkpoint_every, nodes, target)
    loss.backward()   # v0.grad, mu.grad from the hand-written adjoint kernels

`fit_initial_state` fits the initial velocities and the viscosity of a
rollout to a target density field with Adam.
"""
from __future__ import annotations

import numpy as np
import torch

from .solver import Grid, Solver


class DensityFieldLoss(torch.autograd.Function):
    """L(v0, mu) = mean_n (G_n(x_T) - target_n)^2 of a T-step rollout."""

    @staticmethod
    def forward(ctx, v0, mu, solver: Solver, dt: float, steps: int, checkpoint_every: int,
                nodes, target):
        v = v0.detach().to("cpu", torch.float32).numpy()
        solver.rollout_forward(v, float(mu.detach().cpu()), dt, steps, checkpoint_every)
        t = np.ascontiguousarray(target.detach().to("cpu", torch.float32).numpy()
                                 if torch.is_tensor(target) else target, np.float32)
        _, loss = solver.rollout_density_loss(nodes, t)
        ctx.solver = solver
        ctx.v_meta = (v0.device, v0.dtype)
        ctx.mu_meta = (mu.device, mu.dtype)
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        gv, _, gmu = ctx.solver.rollout_backward()
        g = float(grad_out)
        dv, tv = ctx.v_meta
        dm, tm = ctx.mu_meta
        grad_v = torch.from_numpy(gv * np.float32(g)).to(dv, tv)
        grad_mu = torch.tensor(gmu * g, dtype=tm, device=dm)
        return grad_v, grad_mu, None, None, None, None, None, None


def node_grid(dims=(32, 32, 32)):
    """Cell-centre nodes of a grid over the unit box."""
    return Grid.make_grid_dims((0.0, 0.0, 0.0), dims, 1.0 / dims[0])


def fit_initial_state(solver: Solver, target, dt: float, steps: int, iters: int = 10,
                      mu0: float = 2.5, lr_v: float = 0.02, lr_mu: float = 0.5,
                      checkpoint_every: int = 20, nodes=None):
    """Adam on (v0, log mu) starting from v0 = 0, mu = mu0; returns the history."""
    nodes = node_grid() if nodes is None else nodes
    v0 = torch.zeros((solver.num_fluid, 3), dtype=torch.float32, requires_grad=True)
    log_mu = torch.tensor(float(np.log(mu0)), dtype=torch.float64, requires_grad=True)
    opt = torch.optim.Adam([{"params": [v0], "lr": lr_v}, {"params": [log_mu], "lr": lr_mu}])
    hist = []
    for _ in range(iters):
        opt.zero_grad()
        loss = DensityFieldLoss.apply(v0, log_mu.exp(), solver, dt, steps, checkpoint_every,
                                      nodes, target)
        loss.backward()
        opt.step()
        hist.append({"loss": float(loss.detach()), "mu": float(log_mu.detach().exp())})
    return hist, v0.detach(), float(log_mu.detach().exp())
