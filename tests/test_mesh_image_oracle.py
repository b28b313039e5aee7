"""Oracle restatements of the mesh hygiene of meshGenerateBase* and of the
texture post-processing (project definitions; cage is absent), on small
known cases. The GPU path is compared with these in test_gpu_mesh_image.py."""
from __future__ import annotations

import numpy as np


def test_largest_component_and_tie(O):
    # a tetrahedron (4 triangles) and a lone triangle: the tetrahedron stays
    idx = np.array([0, 1, 2, 0, 2, 3, 0, 3, 1, 1, 3, 2, 4, 5, 6], np.uint32)
    pos = np.arange(21, dtype=np.float32).reshape(7, 3)
    p, _, i = O.mesh_filter(pos, None, idx)
    assert p.shape == (4, 3) and np.array_equal(p, pos[:4])
    assert np.array_equal(i, idx[:12])
    # equal sizes: the component holding the lowest vertex index stays
    idx2 = np.array([3, 4, 5, 0, 1, 2], np.uint32)
    p, _, i = O.mesh_filter(pos[:6], None, idx2)
    assert np.array_equal(p, pos[:3]) and np.array_equal(i, [0, 1, 2])
    # isolated vertices (no triangle) are their own, empty components
    p, _, i = O.mesh_filter(pos, None, idx[:12])
    assert p.shape == (4, 3)


def test_water_filter_strip(O):
    # a strip of triangles (i, i+1, i+2): validity spreads two triangles each way
    n = 12
    idx = np.array([[i, i + 1, i + 2] for i in range(n - 2)], np.uint32).reshape(-1)
    pos = np.zeros((n, 3), np.float32)
    pos[:, 0] = np.arange(n)
    valid = np.zeros(n, np.uint8)
    valid[6] = 1
    p, _, i = O.mesh_filter(pos, None, idx, valid=valid)
    # pass 1: triangles 4,5,6 hold vertex 6 -> vertices 4..8; pass 2: triangles 2..8 -> vertices 2..10
    assert np.array_equal(p[:, 0], np.arange(2, 11))
    # kept triangles: all three vertices valid -> triangles 2..8 (first vertex 2..8)
    assert np.array_equal(i.reshape(-1, 3)[:, 0], np.arange(0, 7))


def test_images(O):
    sp = np.random.default_rng(0).integers(0, 256, size=(5, 7, 2), dtype=np.uint8)
    pbr = O.special_to_gltf_pbr(sp)
    assert (pbr[..., 0] == 255).all() and np.array_equal(pbr[..., 1:], sp)
    flat = np.full((6, 9), 77, np.uint8)
    assert (O.height_to_normal(flat) == [128, 128, 255]).all()
    # a ramp along x rising 255 per texel with strength 1: n = (-1, 0, 1)/sqrt(2)
    ramp = np.tile(np.array([0, 255], np.uint8), (3, 1))
    nm = O.height_to_normal(ramp)
    want = np.floor(np.clip(np.array([-1, 0, 1]) / np.sqrt(2) * 0.5 + 0.5, 0, 1) * 255 + 0.5)
    assert (nm == want).all()
