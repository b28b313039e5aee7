"""The allocation-free adjoint entry point, through the C ABI.

up_sdf_param_backward_noalloc serves callers that cannot allocate device
memory (an engine that hands out all device memory from its own pool, or a
process that must not grow its device footprint after start-up): it takes
device buffers only and keeps its scratch in a static device array. This
file is collected last so that a run stopping at the first failure has run
every other test before it; it also passes alone in a fresh process.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import workloads

pytestmark = pytest.mark.gpu


def test_noalloc_adjoint_matches_allocating_entry_point(cuda, up):
    torch = cuda
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    planet = up.Planet(program=P)
    x = np.random.default_rng(21).uniform(-1.4, 1.4, size=(200000, 3)).astype(np.float32)
    d = planet.sdf_points(x)
    w = (2.0 * d / len(d)).astype(np.float32)
    xt = torch.from_numpy(x).cuda()
    wt = torch.from_numpy(w).cuda()
    nt = len(W.theta_of(P))
    ref = torch.empty(nt, device="cuda")
    assert planet.lib.up_sdf_param_backward(planet.h, xt.data_ptr(), len(x), wt.data_ptr(), ref.data_ptr()) == 0
    ref = ref.cpu().numpy()
    tol = 1e-3 * np.abs(ref).max()   # the adjoint tests' tolerance
    for _ in range(2):                # two calls in a row share the static scratch
        out = torch.full((nt,), float("nan"), device="cuda")
        st = planet.lib.up_sdf_param_backward_noalloc(planet.h, xt.data_ptr(), len(x), wt.data_ptr(), out.data_ptr())
        assert st == 0, planet.lib.up_last_error(planet.h)
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert np.abs(got - ref).max() <= tol


def test_noalloc_adjoint_rejects_host_buffers(cuda, up):
    W = workloads()
    planet = up.Planet(program=W.sphere_fbm())
    x = np.zeros((16, 3), np.float32)
    w = np.ones(16, np.float32)
    out = np.zeros(9, np.float32)
    st = planet.lib.up_sdf_param_backward_noalloc(planet.h, x.ctypes.data, 16, w.ctypes.data, out.ctypes.data)
    assert st == up.abi.UP_ERR_INVALID_ARGUMENT
    assert b"device buffers" in planet.lib.up_last_error(planet.h)
