"""The |n| bounds of the gradient noises used by the narrow band of
contouring (noise_abs_bound in csrc/up_synth.cuh: 1.1 for Perlin, simplex
and simplex-reduced).

|g.d| <= max over axis pairs (|d_a| + |d_b|) for every 12-edge gradient g,
so |n(p)| <= M(p) = sum over the corners of the kernel weight times that
maximum. M is evaluated on a dense grid of the cell (of the skewed cell for
simplex), and its maximum plus the largest change between grid neighbours
(a bound on the variation inside a grid cell, doubled) must stay below 1.1."""
from __future__ import annotations

import numpy as np

BOUND = 1.1


def _pairmax(dx, dy, dz):
    ax, ay, az = np.abs(dx), np.abs(dy), np.abs(dz)
    return np.maximum(np.maximum(ax + ay, ax + az), ay + az)


def _check(M, h):
    slope = max(np.abs(np.diff(M, axis=a)).max() for a in range(3))
    assert M.max() + 2 * slope <= BOUND, (M.max(), slope)


def test_perlin_majorant():
    h = 1 / 120
    t = np.arange(0, 1 + 1e-9, h)
    fx, fy, fz = np.meshgrid(t, t, t, indexing="ij")
    fade = lambda u: u * u * u * (u * (u * 6 - 15) + 10)  # noqa: E731
    M = np.zeros_like(fx)
    for cx in (0, 1):
        for cy in (0, 1):
            for cz in (0, 1):
                w = (fade(fx) if cx else 1 - fade(fx)) * (fade(fy) if cy else 1 - fade(fy)) * (fade(fz) if cz else 1 - fade(fz))
                M += w * _pairmax(fx - cx, fy - cy, fz - cz)
    assert M.max() > 1.0  # the bound is not loose by much
    _check(M, h)


def _simplex_offsets(h):
    g3 = 1 / 6
    t = np.arange(0, 1, h) + h / 2
    xs, ys, zs = np.meshgrid(t, t, t, indexing="ij")
    tt = (xs + ys + zs) * g3
    x0, y0, z0 = xs - tt, ys - tt, zs - tt
    # second and third corners by the rank order of the offsets (Gustavson)
    rx = (x0 >= y0).astype(int) + (x0 >= z0).astype(int)
    ry = (y0 > x0).astype(int) + (y0 >= z0).astype(int)
    rz = (z0 > x0).astype(int) + (z0 > y0).astype(int)
    i1, j1, k1 = (rx >= 2), (ry >= 2), (rz >= 2)
    i2, j2, k2 = (rx >= 1), (ry >= 1), (rz >= 1)
    return [(x0, y0, z0), (x0 - i1 + g3, y0 - j1 + g3, z0 - k1 + g3), (x0 - i2 + 2 * g3, y0 - j2 + 2 * g3, z0 - k2 + 2 * g3),
            (x0 - 1 + 3 * g3, y0 - 1 + 3 * g3, z0 - 1 + 3 * g3)]


def test_simplex_majorants():
    h = 1 / 100
    offs = _simplex_offsets(h)
    for power, scale in ((4, 76.0), (3, 31.0)):
        M = np.zeros_like(offs[0][0])
        for dx, dy, dz in offs:
            tc = np.maximum(0.5 - dx * dx - dy * dy - dz * dz, 0.0)
            M += scale * tc ** power * _pairmax(dx, dy, dz)
        assert M.max() > 0.95
        _check(M, h)
