"""PyTorch binding: the projection step as a differentiable operator.

``ProjectionFn`` wraps covof_projection_dev (Poisson solve on -div u*, then
u = u* - dt/rho grad p) and, in backward, covof_projection_vjp_dev: one
adjoint Poisson solve with the same symmetric operator plus a face kernel,
giving gradients with respect to the predicted velocity u* and the face
coefficients beta = 1/rho_face.  Tensors are float64 CUDA tensors in the
reference layout (ny+2, nx+2).  The geometric VOF step is not differentiable
and has no binding here.
"""
from __future__ import annotations

import torch

from .solver import Solver


def _c(t):
    return t.contiguous() if t is not None else None


class ProjectionFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u_star, v_star, beta_u, beta_v, solver: Solver, dt: float):
        for t in (u_star, v_star, beta_u, beta_v):
            if t.dtype != torch.float64 or not t.is_cuda:
                raise TypeError("ProjectionFn expects float64 CUDA tensors")
        u_star, v_star = _c(u_star), _c(v_star)
        one = torch.ones((), dtype=torch.float64, device=u_star.device)
        rho_u = torch.where(beta_u > 0, one / beta_u, one).contiguous()
        rho_v = torch.where(beta_v > 0, one / beta_v, one).contiguous()
        p = torch.zeros_like(u_star)
        u = torch.empty_like(u_star)
        v = torch.empty_like(v_star)
        torch.cuda.current_stream().synchronize()  # the library runs on its own stream
        solver.projection_dev(dt, u_star, v_star, rho_u, rho_v, p, u, v)
        ctx.save_for_backward(rho_u, rho_v, p)
        ctx.solver, ctx.dt = solver, dt
        return u, v, p

    @staticmethod
    def backward(ctx, gu, gv, gp):
        rho_u, rho_v, p = ctx.saved_tensors
        gu = _c(gu) if gu is not None else torch.zeros_like(p)
        gv = _c(gv) if gv is not None else torch.zeros_like(p)
        gp = _c(gp)
        outs = [torch.zeros_like(p) for _ in range(4)]
        torch.cuda.current_stream().synchronize()
        ctx.solver.projection_vjp_dev(ctx.dt, rho_u, rho_v, p, gu, gv, gp, *outs)
        return outs[0], outs[1], outs[2], outs[3], None, None


def project(u_star, v_star, beta_u, beta_v, solver: Solver, dt: float):
    """Differentiable projection: returns (u, v, p)."""
    return ProjectionFn.apply(u_star, v_star, beta_u, beta_v, solver, dt)
