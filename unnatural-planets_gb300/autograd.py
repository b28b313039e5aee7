"""torch.autograd.Function over the C-ABI SDF of a synthetic planet.

SynthSDF.apply(theta, points, planet) returns d(points; theta) (FP32, on
the points' device); SynthSDFGrid does the same for every sample of a grid
through the grid kernel. Its backward calls the library's hand-written adjoint
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


class SynthSDFGrid(torch.autograd.Function):
    """d on every sample of a grid (x fastest, grid.count values) from the
    x-coherent grid kernel (up_sdf_grid). Its backward is SynthSDF's at the
    grid's sample positions (grid_positions: the kernels' coordinates)."""
    @staticmethod
    def forward(ctx, theta: torch.Tensor, grid, planet, positions: torch.Tensor):
        th = theta.detach().to(torch.float32).contiguous().cpu()
        planet.set_theta(th.numpy())
        d = torch.empty(grid.count, dtype=torch.float32, device=positions.device)
        planet.sdf_grid(grid, 1, outs=[d, None, None])
        ctx.planet = planet
        ctx.save_for_backward(positions)
        ctx.theta_dtype = theta.dtype
        return d

    @staticmethod
    def backward(ctx, dL_dd: torch.Tensor):
        (pts,) = ctx.saved_tensors
        w = dL_dd.detach().to(torch.float32).contiguous()
        dth = torch.empty(len(_theta_of(ctx.planet)), dtype=torch.float32, device=pts.device)
        ctx.planet.param_backward(pts, w, dtheta=dth)
        return dth.to(ctx.theta_dtype), None, None, None


def grid_positions(grid, device="cuda") -> torch.Tensor:
    """(count, 3) FP32 sample positions of a grid, x fastest, computed as the
    kernels compute them: step = (hi - lo) / (n - 1), x_i = i * step + lo
    (a rounded product, then a rounded sum)."""
    ax = []
    for a in range(3):
        lo = torch.tensor(float(grid.lo[a]), dtype=torch.float32, device=device)
        hi = torch.tensor(float(grid.hi[a]), dtype=torch.float32, device=device)
        step = (hi - lo) / torch.tensor(float(int(grid.n[a]) - 1), dtype=torch.float32, device=device)
        i = torch.arange(int(grid.n[a]), dtype=torch.float32, device=device)
        ax.append((i * step) + lo)
    zz, yy, xx = torch.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return torch.stack([xx.reshape(-1), yy.reshape(-1), zz.reshape(-1)], dim=1).contiguous()


class RelativeTheta(torch.nn.Module):
    """theta = theta0 * (1 + scale * u), with u the parameter an optimiser moves.

    The program's parameters span five orders of magnitude (octave amplitudes
    of 6e-4, frequencies up to 96, radii near 1). An optimiser step of fixed
    size in theta overshoots the small ones and barely moves the large ones;
    in u every parameter moves in units of its own starting size. Entries of
    theta0 that are 0 cannot move.

    scale (default 1) sets each parameter's unit further. With
    workloads.phase_scale a frequency f moves in units of f_min / f of itself:
    one unit shifts every octave's noise by the same number of lattice cells
    at a given point. The loss is only locally convex in a frequency (the
    noise at p decorrelates once the frequency error times |p| reaches about
    one cell, 0.7 % at f = 96 and |p| = 1.4), so equal relative steps (an Adam
    step of lr = 1e-2 moves every u by about 1e-2) throw the high octaves out
    of their basins in the first steps."""

    def __init__(self, theta0: torch.Tensor, scale: torch.Tensor | None = None):
        super().__init__()
        self.register_buffer("theta0", theta0.detach().clone())
        s = torch.ones_like(self.theta0) if scale is None else scale.detach().to(self.theta0).clone()
        self.register_buffer("scale", s)
        self.u = torch.nn.Parameter(torch.zeros_like(self.theta0))

    def forward(self) -> torch.Tensor:
        return self.theta0 * (1 + self.scale * self.u)


def _theta_of(planet):
    from .workloads import theta_of
    return theta_of(planet.program)


def sdf(theta, points, planet):
    return SynthSDF.apply(theta, points, planet)


def sdf_grid(theta, grid, planet, positions=None):
    """d on the grid's samples (flat, x fastest); positions: grid_positions(grid), reused across calls"""
    if positions is None:
        positions = grid_positions(grid)
    return SynthSDFGrid.apply(theta, grid, planet, positions)
