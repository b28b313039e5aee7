"""up_mesh_generate_base (largest component, water filter, ordered
compaction) and the texture post-processing (up_image_*) against the
oracle's restatements.

The oracle filters the GPU's own up_contour mesh of the same grid, and the
water test gives it the validity computed from the GPU's elevationRaw at
those vertices (the same points kernel the library uses), so kept vertices
and triangles must match bit for bit. Normal maps: within 1 level (FP32 on
the GPU, FP64 in the oracle)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu


def _check_same(got, want):
    gp, gn, gi = got
    wp, wn, wi = want
    assert np.array_equal(gi, wi)
    assert np.array_equal(gp, wp)
    if wn is not None:
        assert np.array_equal(gn, wn)


def test_base_mesh_synthetic_largest_component(cuda, up, O):
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    g = W.grid(W.GRID_C2, n=(96, 96, 96))
    planet = up.Planet(program=P)
    pos, nrm, idx = planet.contour(g)
    want = O.mesh_filter(pos, nrm, idx)
    got = planet.mesh_generate_base(g)
    _check_same(got, want)
    # the spheres outside the torus band are separate components: some geometry goes
    assert len(want[2]) < len(idx) and len(want[0]) < len(pos)


def test_base_mesh_from_values_and_device_buffers(cuda, up, O):
    torch = cuda
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    g = W.grid(W.GRID_C2, n=(64, 64, 64))
    planet = up.Planet(program=P)
    vals = planet.sdf_grid(g, 1)[0]
    want = planet.mesh_generate_base(g)
    got = planet.mesh_generate_base(g, values=vals)
    _check_same(got, want)
    # device output buffers, capacity protocol
    import ctypes as C
    V, I = len(want[0]), len(want[2])
    dp = torch.empty((V, 3), device="cuda")
    di = torch.empty(I, dtype=torch.int32, device="cuda")
    small = up.abi.MeshOut(dp.data_ptr(), None, di.data_ptr(), V - 1, I, 0, 0)
    assert planet.lib.up_mesh_generate_base(planet.h, 0, C.byref(g), None, C.byref(small)) == up.abi.UP_ERR_CAPACITY
    assert small.vertex_count == V and small.index_count == I
    m = up.abi.MeshOut(dp.data_ptr(), None, di.data_ptr(), V, I, 0, 0)
    assert planet.lib.up_mesh_generate_base(planet.h, 0, C.byref(g), None, C.byref(m)) == 0
    assert np.array_equal(dp.cpu().numpy(), want[0])
    assert np.array_equal(di.cpu().numpy().view(np.uint32), want[2])


@pytest.mark.parametrize("shape,elevation,seed", [("sphere", "lakes", 3), ("torus", "islands", 5)])
def test_base_mesh_water_filter(cuda, up, O, shape, elevation, seed):
    planet = up.Planet(shape, elevation, "default", seed=seed)
    g = up.abi.Grid.make((-2000, -2000, -2000), (2000, 2000, 2000), (72, 72, 72))
    pos, nrm, idx = planet.contour(g, field=up.abi.FIELD_WATER)
    elev = planet.sdf_points(pos, field=up.abi.FIELD_ELEVATION_RAW)
    valid = (elev < np.float32(0.1)).astype(np.uint8)
    want = O.mesh_filter(pos, nrm, idx, valid=valid)
    got = planet.mesh_generate_base(g, field=up.abi.FIELD_WATER)
    _check_same(got, want)
    # land and navigation: largest component only
    for f in (up.abi.FIELD_LAND, up.abi.FIELD_NAVIGATION):
        p, n, i = planet.contour(g, field=f)
        _check_same(planet.mesh_generate_base(g, field=f), O.mesh_filter(p, n, i))


def test_images_match_oracle(cuda, up, O):
    torch = cuda
    planet = up.Planet(program=workloads().sphere_fbm())
    r = np.random.default_rng(4)
    sp = r.integers(0, 256, size=(37, 53, 2), dtype=np.uint8)
    assert np.array_equal(planet.special_to_gltf_pbr(sp), O.special_to_gltf_pbr(sp))
    # a smooth height field plus noise, odd sizes, both strengths
    y, x = np.mgrid[0:61, 0:47]
    h = np.clip(127 + 90 * np.sin(x / 7.0) * np.cos(y / 5.0) + r.normal(0, 6, size=x.shape), 0, 255).astype(np.uint8)
    for s in (1.0, 4.0):
        got = planet.height_to_normal(h, strength=s)
        want = O.height_to_normal(h, strength=s)
        assert np.abs(got.astype(int) - want.astype(int)).max() <= 1
    # device buffers in and out
    hd = torch.from_numpy(h).cuda()
    od = torch.empty((61, 47, 3), dtype=torch.uint8, device="cuda")
    assert planet.lib.up_image_height_to_normal(planet.h, hd.data_ptr(), 47, 61, 1.0, od.data_ptr()) == 0
    assert np.array_equal(od.cpu().numpy(), planet.height_to_normal(h))
    # single-texel rows and columns
    assert np.array_equal(planet.height_to_normal(h[:1]), O.height_to_normal(h[:1]))
    col = np.ascontiguousarray(h[:, :1])
    assert np.abs(planet.height_to_normal(col).astype(int) - O.height_to_normal(col).astype(int)).max() <= 1
