"""Parity at the benchmark configurations' own sizes, through the C ABI,
against the FP64 oracle (reference rows: the SDF value of
modesConfiguration.cpp:248-258, the grid and mesh of meshGeneration.cpp:19-44,
the texels of textures.cpp:24-43).

  plain method   sphere - 4-octave simplex FBM on its 128^3 grid: every
                 sample's value and gradient, and the mesh
  at scale       torus + 8 spheres - ridged Perlin + cellular on its 512^3
                 grid: a seeded sample of 2^20 grid points of the real
                 up_sdf_grid output (value and gradient), and the planet's
                 mesh (up_contour, narrow-band sampling) against the oracle's
                 contouring of the value-only GPU grid
  atlas          the 4096^2 texel atlas of that mesh, every texel

Tolerances (the path's accuracy bar, written here):
  SDF value      |GPU - FP64| <= 1e-5 (unit-scale planets) for every checked sample
  gradient       |GPU - FP64| <= 1e-4 max(1, |grad|) for all but 1e-4 of the
                 samples (cellular F1/F2 swaps and the ridged |n| kink are
                 discontinuities where FP32 and FP64 may take opposite sides)
  topology       triangle indices bit-exact (hence active cells, sign edges
                 and quads too)
  vertices       within 1e-3 of a cell for 99.9 % of them (FP32 Hermite data
                 and QEF against FP64), always inside the cell
  texels         coverage bit-exact; 8-bit channels within 2 levels for
                 99.5 % of covered texels (biome-free synthetic program:
                 value noise, simplex noise, height)
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu

VALUE_TOL = 1e-5
GRAD_TOL = 1e-4
GRAD_OUTLIERS = 1e-4


def _grad_outliers(g, g64):
    e = np.abs(np.asarray(g, np.float64) - g64).max(axis=1) / np.maximum(1.0, np.abs(g64).max(axis=1))
    return (e > GRAD_TOL).mean()


def _vertex_check(pos, ref_pos, step):
    err = (np.abs(pos.astype(np.float64) - ref_pos) / step).max(axis=1)
    assert (err > 1e-3).mean() <= 1e-3, (err > 1e-3).mean()
    assert err.max() <= 1.0


def test_plain_method_128(cuda, up, O):
    W = workloads()
    P = W.sphere_fbm()
    g = W.grid(W.GRID_C1)
    assert tuple(g.n) == (128, 128, 128)
    planet = up.Planet(program=P)
    n = g.count
    d = np.empty(n, np.float32)
    grad = np.empty(3 * n, np.float32)
    planet.sdf_grid(g, 1, outs=[d, None, None], grad=grad)
    ref, rg = O.synth_points(P, O.grid_positions(g), grad=True, threads=16)
    assert np.abs(d - ref).max() <= VALUE_TOL
    assert _grad_outliers(grad.reshape(3, n).T, rg) <= GRAD_OUTLIERS
    # the mesh: up_contour samples its own grid (narrow band, value-only form)
    # and contours it; the same triangles as contouring the value-only grid
    dp = np.empty(n, np.float32)
    planet.sdf_grid(g, 1, outs=[dp, None, None])
    assert np.abs(d - dp).max() <= 1e-6
    pos, nrm, idx = planet.contour(g)
    mesh = O.contour_synth(P, g, dp)
    assert np.array_equal(idx, mesh["indices"])
    step = (np.asarray(W.GRID_C1["hi"]) - np.asarray(W.GRID_C1["lo"])) / 127
    _vertex_check(pos, mesh["positions"], step)
    assert (np.abs(nrm - mesh["normals"]).max(axis=1) > 1e-3).mean() <= 1e-3


@pytest.fixture(scope="module")
def planet512(cuda, up, O):
    """The 512^3 benchmark planet: the value-only grid (host copy), a 2^20
    sample of grid points with the fused kernel's values and gradients, the
    largest difference between the fused and value-only values, and the
    planet's mesh from up_contour."""
    torch = cuda
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    g = W.grid(W.GRID_C2)
    assert tuple(g.n) == (512, 512, 512)
    n = g.count
    planet = up.Planet(program=P)
    d = torch.empty(n, device="cuda")
    gr = torch.empty(3 * n, device="cuda")
    planet.sdf_grid(g, 1, outs=[d, None, None], grad=gr)
    idx = np.unique(np.random.default_rng(2024).integers(0, n, size=1 << 20, dtype=np.int64))
    it = torch.from_numpy(idx).cuda()
    dv = d[it].cpu().numpy()
    gv = torch.stack([gr[it], gr[n + it], gr[2 * n + it]], dim=1).cpu().numpy()
    del gr
    dp = torch.empty(n, device="cuda")
    planet.sdf_grid(g, 1, outs=[dp, None, None])
    fused_vs_plain = float((d - dp).abs().max())
    del d
    values = dp.cpu().numpy()
    del dp
    pos, nrm, tri = planet.contour(g)
    return dict(P=P, g=g, planet=planet, idx=idx, dv=dv, gv=gv, values=values, pos=pos, nrm=nrm, tri=tri,
                fused_vs_plain=fused_vs_plain)


def test_at_scale_512_values(planet512, O):
    s = planet512
    x = O.grid_positions_at(s["g"], s["idx"])
    ref, rg = O.synth_points(s["P"], x, grad=True, threads=16)
    # fused and value-only forms agree to FP32 rounding over the whole grid
    assert s["fused_vs_plain"] <= 1e-6
    assert np.abs(s["dv"] - s["values"][s["idx"]]).max() <= 1e-6
    assert np.abs(s["dv"] - ref).max() <= VALUE_TOL
    assert np.abs(s["values"][s["idx"]] - ref).max() <= VALUE_TOL
    assert _grad_outliers(s["gv"], rg) <= GRAD_OUTLIERS


def test_at_scale_512_mesh(planet512, O):
    """The planet's mesh (narrow-band sampling inside up_contour) against the
    oracle's contouring of the exactly sampled value-only GPU grid: the same
    triangles (the narrow band changes no sign that contouring reads)."""
    s = planet512
    W = workloads()
    mesh = O.contour_synth(s["P"], s["g"], s["values"])
    assert len(s["pos"]) == len(mesh["positions"])
    assert np.array_equal(s["tri"], mesh["indices"])
    step = (np.asarray(W.GRID_C2["hi"]) - np.asarray(W.GRID_C2["lo"])) / 511
    _vertex_check(s["pos"], mesh["positions"], step)


def test_at_scale_atlas_4096(planet512, O):
    s = planet512
    W = workloads()
    p2, n2, uv, i2 = W.quad_atlas(s["pos"], s["nrm"], s["tri"], 4096, 4096)
    got = s["planet"].texture(1, p2, n2, uv, i2, 4096, 4096, dilation=7, floats=True)
    want = O.texture(1, p2, n2, uv, i2, 4096, 4096, dilation=7, program=s["P"], threads=16)
    assert np.array_equal(np.isnan(got["height_f"]), np.isnan(want["height_f"]))
    covered = want["owner"] >= 0
    assert covered.mean() > 0.3   # 4 x 4 texel charts with half a texel of margin
    for k in ("albedo", "special", "height"):
        diff = np.abs(got[k].astype(int) - want[k].astype(int))
        if diff.ndim == 3:
            diff = diff.max(axis=2)
        assert (diff[covered] > 2).mean() <= 5e-3, k
