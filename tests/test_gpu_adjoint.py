"""GPU parameter adjoint (up_sdf_param_backward) against the oracle's
forward-mode FP64 gradient: relative 1e-3 of the largest entry."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["c1", "c2"])
def test_param_backward(cuda, up, O, which):
    W = workloads()
    P = W.sphere_fbm() if which == "c1" else W.torus_spheres_ridged_cellular()
    x = W.shell_points(1.0, 0.05, 50000, seed=7) if which == "c1" else \
        np.random.default_rng(8).uniform(-1.4, 1.4, size=(50000, 3)).astype(np.float32)
    planet = up.Planet(program=P)
    d = planet.sdf_points(x)
    w = (2.0 * d / len(d)).astype(np.float32)   # dL/dd of L = mean(d^2)
    dt = planet.param_backward(x, w)
    ref = O.synth_theta_grad(P, x, w.astype(np.float64))
    assert np.abs(dt - ref).max() <= 1e-3 * np.abs(ref).max()
    # deterministic: same result twice, bit for bit
    assert np.array_equal(planet.param_backward(x, w), dt)


def _shell_points(planet, n, seed, half_width=0.05):
    """n points uniform in {|d| < half_width} of the torus program (rejection
    from the box)."""
    rng = np.random.default_rng(seed)
    got = []
    while sum(len(p) for p in got) < n:
        c = rng.uniform(-1.6, 1.6, size=(200000, 3)).astype(np.float32)
        got.append(c[np.abs(planet.sdf_points(c)) < half_width])
    return np.concatenate(got)[:n]


def test_torus_adjoint_vs_fp64_central_differences(cuda, up, O):
    """The adjoint of L = mean(d^2) for the 25 parameters of the torus +
    spheres - ridged Perlin + cellular planet against FP64 central
    differences (h = 1e-4) of the oracle's L, on 4096 seeded points of the
    0.05 shell."""
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    planet = up.Planet(program=P)
    x = _shell_points(planet, 4096, seed=21)
    d = planet.sdf_points(x)
    w = (2.0 * d / len(d)).astype(np.float32)
    dt = planet.param_backward(x, w)
    th = O.synth_theta(P)
    assert len(th) == len(dt) == 25
    h = 1e-4
    cd = np.empty_like(th)
    for i in range(len(th)):
        tp, tm = th.copy(), th.copy()
        tp[i] += h
        tm[i] -= h
        cd[i] = (np.mean(O.synth_points(P, x, theta=tp) ** 2) - np.mean(O.synth_points(P, x, theta=tm) ** 2)) / (2 * h)
    assert np.abs(dt - cd).max() <= 2e-3 * np.abs(cd).max()
