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
