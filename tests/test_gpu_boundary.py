"""The drop-in boundary under the reference's conditions, through the C ABI:
the per-point terrain callbacks called from many threads at once (the
reference runs its navmesh, land and water pipelines and their chunk tasks
concurrently, generator.cpp:159,215,432-439), the ELEVATION field
(modesConfiguration.cpp:230-237), buffers of the context's GPU used in place,
and the out-of-memory status through the host-side allocation fault."""
from __future__ import annotations

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pts(n, seed, lo=-2000.0, hi=2000.0):
    return np.random.default_rng(seed).uniform(lo, hi, size=(n, 3)).astype(np.float32)


@pytest.mark.parametrize("shape,elevation", [("sphere", "lakes"), ("torus", "craters")])
def test_callbacks_from_eight_threads(cuda, up, shape, elevation):
    """8 host threads call up_sdf_land / water / navigation at the same time
    (ctypes releases the GIL for the call); every value equals the batched
    up_sdf_eval_points of the same points bit for bit."""
    planet = up.Planet(shape, elevation, seed=3)
    lib = planet.lib
    assert lib.up_set_current_context(planet.h) == 0
    fns = [lib.up_sdf_land, lib.up_sdf_water, lib.up_sdf_navigation]
    n_threads, n_pts = 8, 160
    pts = [_pts(n_pts, 100 + t) for t in range(n_threads)]
    got = [np.full(n_pts, np.nan, np.float32) for _ in range(n_threads)]
    start = threading.Barrier(n_threads)

    def work(t):
        f = fns[t % 3]
        start.wait()
        for i in range(n_pts):
            got[t][i] = f(pts[t][i].ctypes.data)
    th = [threading.Thread(target=work, args=(t,)) for t in range(n_threads)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    for t in range(n_threads):
        ref = planet.sdf_points(pts[t], field=t % 3)
        assert np.array_equal(ref.view(np.uint32), got[t].view(np.uint32)), t
    # installing another context retires the copies: the callbacks follow it
    other = up.Planet(shape, "none", seed=3)
    assert lib.up_set_current_context(other.h) == 0
    v = lib.up_sdf_land(pts[0][0].ctypes.data)
    assert np.float32(v) == other.sdf_points(pts[0][:1])[0]
    assert lib.up_set_current_context(None) == 0
    assert np.isnan(lib.up_sdf_land(pts[0][0].ctypes.data))


def test_callback_copy_follows_theta(cuda, up, W):
    """up_context_set_theta on the installed synthetic context retires the
    calling threads' copies: the callback sees the new parameters."""
    P = W.sphere_fbm()
    planet = up.Planet(program=P)
    lib = planet.lib
    lib.up_set_current_context(planet.h)
    p = np.array([1.0, 0.2, -0.1], np.float32)
    a = lib.up_sdf_land(p.ctypes.data)
    th = W.theta_of(P).copy()
    th[-1] = 1.25   # sphere radius
    planet.set_theta(th)
    b = lib.up_sdf_land(p.ctypes.data)
    assert np.float32(b) == planet.sdf_points(p[None])[0]
    assert abs((a - b) - 0.25) < 1e-6
    lib.up_set_current_context(None)


@pytest.mark.parametrize("shape", ["sphere", "torus", "mandelbulb", "gear"])
def test_elevation_field(cuda, up, O, shape):
    """UP_FIELD_ELEVATION = shape(p) * 10 (terrainSdfElevation), against the
    FP32 and FP64 oracles, with its gradient."""
    x = _pts(4000, 31)
    planet = up.Planet(shape, "lakes", seed=8)
    d, g = planet.sdf_points(x, field=up.abi.FIELD_ELEVATION, want_grad=True)
    ref = O.Planet(shape, "lakes", seed=8)
    f32 = ref.field(up.abi.FIELD_ELEVATION, x, precision=1)
    f64, g64 = ref.field(up.abi.FIELD_ELEVATION, x, grad=True)
    water = ref.field(up.abi.FIELD_WATER, x)
    assert np.allclose(f64, 10.0 * water, rtol=1e-12, atol=1e-9)   # the definition
    scale = 10.0 * 1100.0   # shape scale of the reference's planets, times 10
    assert (np.abs(d - f32) > 1e-5 * scale).mean() <= 1e-3
    assert (np.abs(d - f64) > 1e-5 * scale).mean() <= 1e-3
    ge = np.abs(g - g64).max(axis=1) / np.maximum(10.0, np.abs(g64).max(axis=1))
    assert (ge > 1e-3).mean() <= 1e-2


def test_device_buffers_used_in_place(cuda, up, W):
    """Device outputs of the context's GPU are written in place: the call
    allocates no staging buffer for them."""
    torch = cuda
    planet = up.Planet(program=W.sphere_fbm())
    x = torch.from_numpy(_pts(4096, 5, -1.3, 1.3)).cuda()
    d = torch.empty(4096, device="cuda")
    g = torch.empty((4096, 3), device="cuda")
    before = planet.lib.up_context_device_bytes(planet.h)
    planet.sdf_points(x, d=d, grad=g, want_grad=True)
    assert planet.lib.up_context_device_bytes(planet.h) == before
    ref, rg = planet.sdf_points(x.cpu().numpy(), want_grad=True)     # host buffers: staged through scratch
    assert planet.lib.up_context_device_bytes(planet.h) > before
    assert np.array_equal(ref, d.cpu().numpy()) and np.array_equal(rg, g.cpu().numpy())


def test_out_of_memory_status(cuda, up, W):
    """The host-side allocation fault makes the next scratch allocation fail:
    the call returns UP_ERR_OOM with a message, the context stays usable."""
    planet = up.Planet(program=W.sphere_fbm())
    x = _pts(1000, 6, -1.3, 1.3)
    planet.lib.up_debug_fail_allocations(1)
    with pytest.raises(up.UpError) as e:
        planet.sdf_points(x)
    assert e.value.status == up.abi.UP_ERR_OOM
    assert b"out of memory" in planet.lib.up_last_error(planet.h)
    d = planet.sdf_points(x)   # the fault was used up
    assert np.all(np.isfinite(d))
    planet.lib.up_debug_fail_allocations(0)
