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
