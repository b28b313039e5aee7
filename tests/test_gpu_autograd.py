"""torch.autograd wrapper over the C-ABI adjoint: gradients against the
oracle's FP64 forward-mode theta gradient, and a short inverse fit (the
benchmark's differentiation workload, scaled down) that recovers a perturbed
parameter vector."""
from __future__ import annotations

import importlib

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu


def test_backward_matches_oracle(cuda, up, O):
    torch = cuda
    AG = importlib.import_module("unnatural-planets_gb300.autograd")
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    planet = up.Planet(program=P)
    x = np.random.default_rng(2).uniform(-1.4, 1.4, size=(40000, 3)).astype(np.float32)
    pts = torch.from_numpy(x).cuda()
    theta = torch.from_numpy(W.theta_of(P)).cuda().requires_grad_(True)
    d = AG.sdf(theta, pts, planet)
    loss = (d * d).mean()
    loss.backward()
    w = 2.0 * d.detach().cpu().numpy().astype(np.float64) / len(x)
    ref = O.synth_theta_grad(P, x, w)
    got = theta.grad.cpu().numpy()
    assert np.abs(got - ref).max() <= 1e-3 * np.abs(ref).max()


def test_inverse_fit_recovers_parameters(cuda, up):
    """The inverse-fit protocol on the plain method's 9 parameters (sphere
    radius, 4 octave amplitudes and 4 frequencies): theta0 = theta* (1 + 0.05 U)
    from a second seed, 300 Adam steps (lr 1e-2) on the relative parameters
    u (theta = theta0 (1 + u)), L = mean((d - d*)^2) over 200,000 points of
    the shell |p| in [0.9, 1.1]. theta is recovered to 0.5 % (measured on
    GB300: ~1e-7 for three seeds)."""
    torch = cuda
    AG = importlib.import_module("unnatural-planets_gb300.autograd")
    W = workloads()
    target = W.sphere_fbm(seed=5)
    t_star = torch.from_numpy(W.theta_of(target)).cuda()
    x = torch.from_numpy(W.shell_points(1.0, 0.1, 200000, seed=9)).cuda()
    planet_t = up.Planet(program=target)
    d_star = planet_t.sdf_points(x, d=torch.empty(x.shape[0], device="cuda"))
    for seed in (6, 7):
        rng = np.random.default_rng(seed)
        t0 = t_star.cpu().numpy() * (1 + 0.05 * rng.uniform(-1, 1, size=t_star.shape[0])).astype(np.float32)
        rel = AG.RelativeTheta(torch.tensor(t0, device="cuda"))
        planet = up.Planet(program=W.sphere_fbm(seed=5))
        opt = torch.optim.Adam(rel.parameters(), lr=1e-2)
        first = None
        for _ in range(300):
            opt.zero_grad()
            loss = ((AG.sdf(rel(), x, planet) - d_star) ** 2).mean()
            loss.backward()
            opt.step()
            first = first if first is not None else float(loss.detach())
        assert float(loss.detach()) < 1e-6 * first
        err = float((rel().detach() - t_star).norm() / t_star.norm())
        assert err < 5e-3, (seed, err)


def test_gradcheck_4096_points(cuda, up):
    """torch.autograd.gradcheck of L(theta) = mean(d(x; theta)^2) on 4096
    seeded shell points of the sphere - 4-octave simplex FBM planet (smooth in
    theta). The SDF computes in FP32, so the finite differences use a large
    step and tolerances set for FP32 rounding."""
    torch = cuda
    AG = importlib.import_module("unnatural-planets_gb300.autograd")
    W = workloads()
    P = W.sphere_fbm()
    planet = up.Planet(program=P)
    x = torch.from_numpy(W.shell_points(1.0, 0.05, 4096, seed=13)).cuda()
    theta = torch.from_numpy(W.theta_of(P)).cuda().requires_grad_(True)

    def loss(t):
        d = AG.sdf(t, x, planet)
        return (d.double() ** 2).mean()

    assert torch.autograd.gradcheck(loss, (theta,), eps=2e-3, atol=2e-5, rtol=2e-2, nondet_tol=1e-6, fast_mode=False)


def test_grid_function_matches_points(cuda, up, O):
    """SynthSDFGrid (forward through the grid kernel) against SynthSDF at the
    same sample positions: grid_positions are the kernels' coordinates (the
    oracle's grid positions bit for bit), the values agree to FP32
    reassociation, and the parameter gradients of a hinge loss (most weights
    zero, skipped by the adjoint) agree with the points form."""
    torch = cuda
    AG = importlib.import_module("unnatural-planets_gb300.autograd")
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    planet = up.Planet(program=P)
    g = W.grid(W.GRID_C2, n=(40, 37, 33))
    pos = AG.grid_positions(g)
    assert np.array_equal(pos.cpu().numpy(), O.grid_positions(g))
    theta = torch.from_numpy(W.theta_of(P)).cuda()
    sign = torch.sign(AG.sdf(theta, pos, planet)).detach()
    t1 = (theta * 1.03).requires_grad_(True)
    t2 = (theta * 1.03).requires_grad_(True)
    dg = AG.sdf_grid(t1, g, planet, pos)
    dp = AG.sdf(t2, pos, planet)
    assert torch.abs(dg - dp).max().item() < 2e-6
    torch.relu(-dg * sign).mean().backward()
    torch.relu(-dp * sign).mean().backward()
    assert (dg * sign < 0).any() and (dg * sign >= 0).float().mean().item() > 0.5  # a hinge with zero and non-zero weights
    np.testing.assert_allclose(t1.grad.cpu().numpy(), t2.grad.cpu().numpy(), rtol=1e-4, atol=1e-7)
