"""GPU dual contouring against the oracle's contouring of the same FP32
grid: topology (active cells, sign edges, triangle indices) bit-exact;
vertex positions within 1e-3 of a cell (FP64 QEF on both sides, Hermite
normals FP32 on the GPU vs FP64 in the oracle) for at least 99.9% of the
vertices -- a Hermite normal taken at a gradient discontinuity (cellular
F1/F2 swap) may come from either side -- and every vertex inside its cell."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which,n", [("c1", (48, 48, 48)), ("c2", (64, 60, 56))])
def test_contour_matches_oracle(cuda, up, O, which, n):
    W = workloads()
    P, spec = (W.sphere_fbm(), W.GRID_C1) if which == "c1" else (W.torus_spheres_ridged_cellular(), W.GRID_C2)
    g = W.grid(spec, n=n)
    planet = up.Planet(program=P)
    d = planet.sdf_grid(g, 1)[0]
    pos, nrm, idx = planet.contour(g)
    ref = O.contour_synth(P, g, d)
    assert len(pos) == len(ref["positions"])
    assert np.array_equal(idx, ref["indices"])
    step = (np.asarray(spec["hi"]) - np.asarray(spec["lo"])) / (np.asarray(n) - 1)
    err = (np.abs(pos - ref["positions"]) / step).max(axis=1)
    assert (err > 1e-3).mean() <= 1e-3, err.max()
    assert err.max() <= 1.0
    assert (np.abs(nrm - ref["normals"]).max(axis=1) > 1e-3).mean() <= 1e-3
    # contouring the device-sampled grid internally gives the same mesh
    pos2, _, idx2 = planet.contour(g, values=None)
    assert np.array_equal(idx2, idx) and np.array_equal(pos2, pos)


def test_sphere_is_closed_genus0(cuda, up, O):
    """DC of a plain sphere: closed 2-manifold with Euler characteristic 2,
    vertices within a small fraction of a cell of the sphere, outward normals."""
    W = workloads()
    P = W.sphere_fbm(amp=0.0)
    g = W.grid(W.GRID_C1, n=(64, 64, 64))
    pos, nrm, idx = up.Planet(program=P).contour(g)
    tri = idx.reshape(-1, 3)
    edges = np.sort(np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]]), axis=1)
    _, counts = np.unique(edges, axis=0, return_counts=True)
    assert np.all(counts == 2)
    V, E, F = len(pos), len(counts), len(tri)
    assert V - E + F == 2
    r = np.linalg.norm(pos, axis=1)
    h = 2.6 / 63
    assert np.abs(r - 1).max() < 0.05 * h
    fn = np.cross(pos[tri[:, 1]] - pos[tri[:, 0]], pos[tri[:, 2]] - pos[tri[:, 0]])
    assert np.all(np.einsum("ij,ij->i", fn, pos[tri].mean(axis=1)) > 0)
    assert np.all(np.einsum("ij,ij->i", nrm, pos) > 0.99 * np.linalg.norm(pos, axis=1))


def test_capacity_and_empty(cuda, up):
    W = workloads()
    planet = up.Planet(program=W.sphere_fbm())
    g = W.grid(W.GRID_C1, n=(32, 32, 32))
    import ctypes as C
    m = up.abi.MeshOut()
    st = planet.lib.up_contour(planet.h, 0, C.byref(g), None, C.byref(m))
    assert st == up.abi.UP_ERR_CAPACITY and m.vertex_count > 0 and m.index_count % 6 == 0
    far = up.abi.Grid.make((3, 3, 3), (4, 4, 4), (8, 8, 8))
    st = planet.lib.up_contour(planet.h, 0, C.byref(far), None, C.byref(m))
    assert st == up.abi.UP_ERR_EMPTY_MESH
    assert b"empty" in planet.lib.up_last_error(planet.h)


def _band_programs():
    W = workloads()
    rng = np.random.default_rng(12)
    progs = [("c1", W.sphere_fbm(), W.grid(W.GRID_C1, n=(96, 90, 84))),
             ("c2", W.torus_spheres_ridged_cellular(), W.grid(W.GRID_C2, n=(128, 120, 112))),
             # ragged work units: nx % 16, ny % 8 and nz % 4 nonzero, rows not 16-byte aligned
             ("c2r", W.torus_spheres_ridged_cellular(), W.grid(W.GRID_C2, n=(131, 117, 103))),
             # x extent a multiple of 16 (sign words written while sampling), samples ending mid-word
             ("c2h", W.torus_spheres_ridged_cellular(), W.grid(W.GRID_C2, n=(112, 117, 103)))]
    for i in range(3):
        P = W.mixed_planet(rng)
        P.layer[0].amp[0] = 0.3  # a wide band
        progs.append((f"mixed{i}", P, W.grid(dict(lo=(-1.6, -1.6, -1.6), hi=(1.6, 1.6, 1.6), n=(80, 80, 80)))))
    return progs


@pytest.mark.parametrize("k", range(7))
def test_narrow_band_contour_equals_full_grid(cuda, up, k):
    """up_contour samples its grid with the narrow band (noise skipped where
    |base| exceeds the noise bound plus one grid step); contouring the exactly
    sampled grid passed in as values gives the same mesh bit for bit, and so
    does the base mesh."""
    name, P, g = _band_programs()[k]
    planet = up.Planet(program=P)
    full = planet.sdf_grid(g, 1)[0]
    banded = planet.contour(g)
    exact = planet.contour(g, values=full)
    for a, b in zip(banded, exact):
        assert np.array_equal(a, b), name
    for a, b in zip(planet.mesh_generate_base(g), planet.mesh_generate_base(g, values=full)):
        assert np.array_equal(a, b), name
