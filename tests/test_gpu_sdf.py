"""GPU parity of SDF sampling through the C ABI against the FP64 oracle.

Tolerance: |d_gpu - d_fp64| <= 1e-5 (unit-scale programs, FP32 arithmetic);
gradients within 1e-4 * max(1, max|grad|), except at gradient
discontinuities (cellular F1/F2 swaps, ridged creases), where FP32 and FP64
may evaluate opposite sides: at most 1e-4 of the samples may differ there.
The oracle evaluates at the exact FP32 sample positions the CUDA path forms."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu


def grad_ok(g, ref):
    tol = 1e-4 * max(1.0, float(np.abs(ref).max()))
    bad = np.abs(np.asarray(g) - ref).max(axis=1) > tol
    return bad.mean() <= 1e-4


def _programs():
    W = workloads()
    return {"c1": (W.sphere_fbm(), W.GRID_C1), "c2": (W.torus_spheres_ridged_cellular(), W.GRID_C2)}


@pytest.mark.parametrize("which", ["c1", "c2"])
def test_grid_value_and_gradient(cuda, up, O, which):
    W = workloads()
    P, spec = _programs()[which]
    g = W.grid(spec, n=(40, 36, 33))
    planet = up.Planet(program=P)
    n = g.count
    d = np.empty(n, np.float32)
    gr = np.empty(3 * n, np.float32)
    planet.sdf_grid(g, 1, outs=[d, None, None], grad=gr)
    pos = O.grid_positions(g)
    ref, rg = O.synth_points(P, pos, grad=True)
    assert np.abs(d - ref).max() <= 1e-5
    gg = gr.reshape(3, n).T
    assert grad_ok(gg, rg)
    # value-only kernel gives the same values
    d2 = planet.sdf_grid(g, 1)[0]
    assert np.abs(d2 - ref).max() <= 1e-5


@pytest.mark.parametrize("which", ["c1", "c2"])
def test_grid_unaligned_device_outputs(cuda, up, O, which):
    """Sample counts that are not a multiple of 4 (gradient planes off 16-byte
    boundaries) and device outputs starting one float into an allocation:
    the grid kernels' vector stores must fall back to scalar stores. (An even
    nx keeps the x = 0 plane, where samples fall on noise lattice points and
    ridged octaves have a gradient kink, out of the grid.)"""
    torch = cuda
    W = workloads()
    P, spec = _programs()[which]
    g = W.grid(spec, n=(42, 35, 33))
    n = g.count
    assert n % 4 != 0
    planet = up.Planet(program=P)
    dbuf = torch.zeros(n + 1, device="cuda")
    gbuf = torch.zeros(3 * n + 1, device="cuda")
    d, gr = dbuf[1:], gbuf[1:]
    planet.sdf_grid(g, 1, outs=[d, None, None], grad=gr)
    ref, rg = O.synth_points(P, O.grid_positions(g), grad=True)
    assert np.abs(d.cpu().numpy() - ref).max() <= 1e-5
    assert grad_ok(gr.cpu().numpy().reshape(3, n).T, rg)
    assert float(dbuf[0]) == 0.0 and float(gbuf[0]) == 0.0


def test_points_host_and_device_buffers(cuda, up, O):
    torch = cuda
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    x = np.random.default_rng(4).uniform(-1.5, 1.5, size=(100003, 3)).astype(np.float32)
    planet = up.Planet(program=P)
    d, g = planet.sdf_points(x, want_grad=True)
    ref, rg = O.synth_points(P, x, grad=True)
    assert np.abs(d - ref).max() <= 1e-5
    assert grad_ok(g, rg)
    xt = torch.from_numpy(x).cuda()
    dt = torch.empty(len(x), device="cuda")
    gt = torch.empty((len(x), 3), device="cuda")
    planet.sdf_points(xt, d=dt, grad=gt, want_grad=True)
    torch.cuda.synchronize()
    assert np.array_equal(dt.cpu().numpy(), d)
    assert np.array_equal(gt.cpu().numpy(), g)


def test_fp32_oracle_agreement(cuda, up, O):
    """The GPU and the per-operation FP32 restatement agree to FP32 rounding."""
    W = workloads()
    P = W.sphere_fbm()
    x = np.random.default_rng(9).uniform(-1.3, 1.3, size=(20000, 3)).astype(np.float32)
    d = up.Planet(program=P).sdf_points(x)
    f32 = O.synth_points(P, x, precision=1)
    assert np.abs(d - f32).max() <= 2e-6


def test_nan_is_reported(cuda, up):
    """A NaN value is reported as UP_ERR_NAN with the reference's message
    (modesConfiguration.cpp:255-256)."""
    W = workloads()
    P = W.sphere_fbm()
    planet = up.Planet(program=P)
    x = np.array([[0.1, 0.2, np.nan], [0.3, 0.1, 0.2]], np.float32)
    with pytest.raises(up.UpError) as e:
        planet.sdf_points(x)
    assert e.value.status == up.abi.UP_ERR_NAN
    assert "invalid land sdf value" in str(e.value)


def test_invalid_arguments(cuda, up):
    W = workloads()
    planet = up.Planet(program=W.sphere_fbm())
    g = up.abi.Grid.make((0, 0, 0), (1, 1, 1), (1, 4, 4))
    with pytest.raises(up.UpError) as e:
        planet.sdf_grid(g, 1)
    assert e.value.status == up.abi.UP_ERR_INVALID_ARGUMENT


def test_host_outputs_pipelined_equal_device(cuda, up):
    """up_sdf_grid into host memory runs in z-slabs with the device-to-host
    copies overlapped; the values and gradients are the single launch's, bit
    for bit (ragged last slab: 157 planes)."""
    torch = cuda
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    g = W.grid(W.GRID_C2, n=(161, 170, 157))
    planet = up.Planet(program=P)
    n = g.count
    dd = torch.empty(n, device="cuda")
    gd = torch.empty(3 * n, device="cuda")
    planet.sdf_grid(g, 1, outs=[dd, None, None], grad=gd)
    dh = np.empty(n, np.float32)
    gh = np.empty(3 * n, np.float32)
    planet.sdf_grid(g, 1, outs=[dh, None, None], grad=gh)
    assert np.array_equal(dh, dd.cpu().numpy()) and np.array_equal(gh, gd.cpu().numpy())
    pinned = torch.empty(n, pin_memory=True)
    planet.sdf_grid(g, 1, outs=[pinned, None, None])
    # the value-only and value+gradient kernels compute the same formulas; the
    # compiler contracts some products into FMAs differently in the two
    # forms, so they agree to FP32 rounding
    assert np.abs(pinned.numpy().astype(np.float64) - dh).max() <= 1e-6
    # reference modes, three fields in one pass
    mp = up.Planet("sphere", "lakes", "default", seed=2)
    gm = up.abi.Grid.make((-2000, -2000, -2000), (2000, 2000, 2000), (170, 161, 163))
    dev = [torch.empty(gm.count, device="cuda") for _ in range(3)]
    mp.sdf_grid(gm, 7, outs=dev)
    host = mp.sdf_grid(gm, 7)
    for a, b in zip(host, dev):
        assert np.array_equal(a, b.cpu().numpy())


@pytest.mark.parametrize("n", [(2, 2, 2), (3, 5, 7), (17, 2, 9), (2, 33, 3)])
def test_tiny_and_ragged_grids(cuda, up, O, n):
    """Grids smaller than one warp task (16 x-samples of 8 x 4 rows) and
    ragged in every axis: values and gradients against the oracle, and
    contouring either succeeds or reports an empty mesh."""
    W = workloads()
    for P in (W.torus_spheres_ridged_cellular(), W.sphere_fbm()):
        g = up.abi.Grid.make((-1.2, -0.9, -1.1), (1.3, 1.0, 0.7), n)
        planet = up.Planet(program=P)
        cnt = g.count
        d = np.empty(cnt, np.float32)
        gr = np.empty(3 * cnt, np.float32)
        planet.sdf_grid(g, 1, outs=[d, None, None], grad=gr)
        ref, rg = O.synth_points(P, O.grid_positions(g), grad=True)
        assert np.abs(d - ref).max() <= 1e-5
        assert np.abs(gr.reshape(3, cnt).T - rg).max() <= 1e-3 * max(1.0, float(np.abs(rg).max()))
        try:
            pos, _, idx = planet.contour(g)
            assert len(idx) % 6 == 0 and (idx < len(pos)).all()
        except up.UpError as e:
            assert e.status == up.abi.UP_ERR_EMPTY_MESH


def test_points_warp_tables_bit_identical(cuda, up):
    """Per-point evaluation shares cellular cell hashes between the lanes of a
    warp when their points are close (cellular_warp). Spatially sorted points
    take that path, shuffled points the per-lane one: values and gradients
    agree bit for bit, and so does the parameter adjoint up to summation
    order; the last warp is partial (n not a multiple of 32)."""
    torch = cuda
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    planet = up.Planet(program=P)
    n = 200_003
    r = np.random.default_rng(31)
    d = r.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    x = (d * r.uniform(0.6, 1.5, size=(n, 1))).astype(np.float32)
    # sort along a coarse 3-D cell order so that neighbours share warps
    cells = np.floor((x + 1.6) / 0.02).astype(np.int64)
    order = np.lexsort((cells[:, 0], cells[:, 1], cells[:, 2]))
    xs = torch.from_numpy(x[order]).cuda()
    xr = torch.from_numpy(x).cuda()
    vs, gs = torch.empty(n, device="cuda"), torch.empty((n, 3), device="cuda")
    vr, gr = torch.empty(n, device="cuda"), torch.empty((n, 3), device="cuda")
    planet.sdf_points(xs, d=vs, grad=gs, want_grad=True)
    planet.sdf_points(xr, d=vr, grad=gr, want_grad=True)
    inv = np.empty(n, np.int64)
    inv[order] = np.arange(n)
    assert np.array_equal(vs.cpu().numpy()[inv], vr.cpu().numpy())
    assert np.array_equal(gs.cpu().numpy()[inv], gr.cpu().numpy())
    nt = len(W.theta_of(P))
    ts, tr = torch.empty(nt, device="cuda"), torch.empty(nt, device="cuda")
    ws = (2.0 / n) * vs
    wr = (2.0 / n) * vr
    planet.param_backward(xs, ws, dtheta=ts)
    planet.param_backward(xr, wr, dtheta=tr)
    np.testing.assert_allclose(ts.cpu().numpy(), tr.cpu().numpy(), rtol=1e-4, atol=1e-6 * float(tr.abs().max()))
