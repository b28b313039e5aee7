"""Parameterisation of the inverse fit (host only): the groups of the theta
layout, the phase scale of the octave frequencies, and RelativeTheta's
per-parameter units."""
from __future__ import annotations

import importlib

import numpy as np

from conftest import workloads


def test_theta_groups_cover_the_layout():
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    g = W.theta_groups(P)
    n = len(W.theta_of(P))
    allidx = sorted(g["amplitudes"] + g["frequencies"] + g["shape"])
    assert allidx == list(range(n))
    # 6 ridged Perlin octaves + 1 cellular octave; torus radii, 8 sphere radii, k
    assert len(g["amplitudes"]) == 7 and len(g["frequencies"]) == 7 and len(g["shape"]) == 11


def test_phase_scale_equal_cell_shift():
    """f_i * s_i is the same for every octave frequency (one unit of u moves
    each octave's noise by the same number of cells); the rest have scale 1."""
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    t = W.theta_of(P)
    s = W.phase_scale(P, t)
    fi = W.theta_groups(P)["frequencies"]
    prod = t[fi] * s[fi]
    assert np.allclose(prod, prod.min(), rtol=1e-6)
    assert np.isclose(prod.min(), np.abs(t[fi]).min())
    rest = [i for i in range(len(t)) if i not in fi]
    assert np.all(s[rest] == 1.0)


def test_relative_theta_scale():
    import torch
    AG = importlib.import_module("unnatural-planets_gb300.autograd")
    t0 = torch.tensor([2.0, 96.0, 0.5])
    s = torch.tensor([1.0, 3.0 / 96.0, 1.0])
    m = AG.RelativeTheta(t0, s)
    assert torch.equal(m(), t0)
    with torch.no_grad():
        m.u.fill_(0.1)
    assert torch.allclose(m(), t0 * (1 + s * 0.1))
    # default: every unit is the parameter's own size
    m1 = AG.RelativeTheta(t0)
    with torch.no_grad():
        m1.u.fill_(0.1)
    assert torch.allclose(m1(), t0 * 1.1)
