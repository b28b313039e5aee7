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


def test_noalloc_adjoint_allocates_nothing(cuda, up):
    """A fresh context that only ever makes allocation-free calls holds no
    device scratch afterwards (the context's scratch counter stays 0), and the
    device's free memory does not move across a warmed-up call (the first
    launch of a kernel may load its code)."""
    torch = cuda
    W = workloads()
    planet = up.Planet(program=W.sphere_fbm())
    x = torch.from_numpy(np.random.default_rng(5).uniform(-1.3, 1.3, size=(50000, 3)).astype(np.float32)).cuda()
    w = torch.full((50000,), 1.0 / 50000, device="cuda")
    out = torch.empty(len(W.theta_of(W.sphere_fbm())), device="cuda")

    def call():
        st = planet.lib.up_sdf_param_backward_noalloc(planet.h, x.data_ptr(), 50000, w.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        assert st == 0, planet.lib.up_last_error(planet.h)
    call()   # warm-up: the first launch of a kernel may load its code
    free0 = torch.cuda.mem_get_info()[0]
    call()
    assert torch.cuda.mem_get_info()[0] == free0
    assert planet.lib.up_context_device_bytes(planet.h) == 0
    assert np.all(np.isfinite(out.cpu().numpy()))


def test_noalloc_adjoint_rejects_host_buffers(cuda, up):
    W = workloads()
    planet = up.Planet(program=W.sphere_fbm())
    x = np.zeros((16, 3), np.float32)
    w = np.ones(16, np.float32)
    out = np.zeros(9, np.float32)
    st = planet.lib.up_sdf_param_backward_noalloc(planet.h, x.ctypes.data, 16, w.ctypes.data, out.ctypes.data)
    assert st == up.abi.UP_ERR_INVALID_ARGUMENT
    assert b"device buffers" in planet.lib.up_last_error(planet.h)
