"""torch.autograd.Function over the C-ABI SDF of a synthetic planet.

SynthSDF.apply(theta, points, planet) returns d(points; theta) (FP32, on
the points' device). Its backward calls the library's hand-written adjoint
(up_sdf_param_backward: octaves recomputed, block partial sums reduced in a
fixed order) for dL/dtheta and the analytic gradient for dL/dpoints. The
forward sets the context's parameter vector from theta, so one Planet serves
every step of a fit.
"""
from __future__ import annotations

import torch


class SynthSDF(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta: torch.Tensor, points: torch.Tensor, planet):
        th = theta.detach().to(torch.float32).contiguous().cpu()
        planet.set_theta(th.numpy())
        pts = points.detach().to(torch.float32).contiguous()
        d = torch.empty(pts.shape[0], dtype=torch.float32, device=pts.device)
        g = torch.empty((pts.shape[0], 3), dtype=torch.float32, device=pts.device) if points.requires_grad else None
        planet.sdf_points(pts, d=d, grad=g, want_grad=g is not None)
        ctx.planet = planet
        ctx.save_for_backward(pts, g if g is not None else torch.empty(0, device=pts.device))
        ctx.theta_dtype = theta.dtype
        return d

    @staticmethod
    def backward(ctx, dL_dd: torch.Tensor):
        pts, g = ctx.saved_tensors
        w = dL_dd.detach().to(torch.float32).contiguous()
        dth = torch.empty(len(_theta_of(ctx.planet)), dtype=torch.float32, device=pts.device)
        ctx.planet.param_backward(pts, w, dtheta=dth)
        dpts = w[:, None] * g if g.numel() else None
        return dth.to(ctx.theta_dtype), dpts, None


def _theta_of(planet):
    from .workloads import theta_of
    return theta_of(planet.program)


def sdf(theta, points, planet):
    return SynthSDF.apply(theta, points, planet)
