"""Oracle self-checks: frozen golden vectors, hand-derived known answers and
derivative consistency. The oracle is the checker of the CUDA path, so it is
pinned first (parity with the reference itself is unpinned: its arithmetic
lives in the absent cage library)."""
from __future__ import annotations

import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import workloads

GOLD = json.loads((Path(__file__).parent / "golden" / "kat.json").read_text())


def test_hash_golden(O):
    L = O.lib()
    for x, h in GOLD["mix32"]:
        assert L.orc_mix32(x) == h
    for x, y, z, k, h in GOLD["lattice_hash"]:
        assert L.orc_lattice_hash(x, y, z, k) == h
    for s, k in GOLD["seed_key"]:
        assert L.orc_seed_key(s) == k


def test_noise_golden(O):
    pts = np.asarray(GOLD["noise_points"], np.float32)
    for key, vals in GOLD["noise"].items():
        if key == "fbm_simplex4":
            got = O.noise(dict(type=3, fractal=1, octaves=4, frequency=0.7, seed=3), pts)
        elif key == "ridged_perlin6":
            got = O.noise(dict(type=2, fractal=2, octaves=6, frequency=0.3, seed=3), pts)
        elif key.startswith("5_"):
            _, d, op = key.split("_")
            got = O.noise(dict(type=5, seed=7, distance=int(d), operation=int(op)), pts)
        else:
            got = O.noise(dict(type=int(key), seed=7), pts)
        np.testing.assert_allclose(got, vals, rtol=0, atol=1e-12, err_msg=key)


def test_synth_golden(O):
    W = workloads()
    sp = np.asarray(GOLD["synth_points"], np.float32)
    np.testing.assert_allclose(O.synth_points(W.sphere_fbm(), sp), GOLD["synth_c1"], atol=1e-12)
    np.testing.assert_allclose(O.synth_points(W.torus_spheres_ridged_cellular(), sp), GOLD["synth_c2"], atol=1e-12)


def test_lattice_zeros_and_values(O):
    """Perlin gradient noise is zero at lattice points; value noise equals the
    lattice hash value there."""
    r = np.random.default_rng(3)
    xi = r.integers(-1000, 1000, size=(500, 3)).astype(np.float32)
    assert np.abs(O.noise(dict(type=2, seed=5), xi)).max() == 0.0
    L = O.lib()
    key = L.orc_seed_key(5)
    v = O.noise(dict(type=0, seed=5), xi)
    for p, got in zip(xi[:50].astype(int), v[:50]):
        h = L.orc_lattice_hash(int(p[0]), int(p[1]), int(p[2]), key)
        assert got == np.float32((h >> 8) * (1.0 / 8388608.0) - 1.0)


@pytest.mark.parametrize("t", [0, 1, 2, 3, 4])
def test_noise_range(O, t):
    x = np.random.default_rng(t).uniform(-40, 40, size=(100000, 3)).astype(np.float32)
    v = O.noise(dict(type=t, seed=11), x)
    assert np.abs(v).max() <= 1.0 + 1e-9
    assert v.std() > 0.15


@pytest.mark.parametrize("t", [0, 1, 2, 3, 4, 5])
def test_noise_gradient_matches_central_differences(O, t):
    """Forward-mode gradient of every noise type against FP64 central
    differences (h = 1e-4) away from cell boundaries."""
    r = np.random.default_rng(10 + t)
    x = r.uniform(-5, 5, size=(400, 3))
    cfg = dict(type=t, seed=9, operation=4, fractal=1, octaves=3, frequency=0.9)
    _, g = O.noise(cfg, x.astype(np.float32), grad=True)
    h = 1e-3
    for a in range(3):
        xp = x.copy(); xp[:, a] += h
        xm = x.copy(); xm[:, a] -= h
        fd = (O.noise(cfg, xp.astype(np.float32)) - O.noise(cfg, xm.astype(np.float32))) / (np.float32(xp[:, a]) - np.float32(xm[:, a]))
        ok = np.abs(fd - g[:, a]) < 2e-2 * (1 + np.abs(g[:, a]))
        # cellular F2-F1 has kinks where the nearest points swap; FD straddles them more often
        assert ok.mean() > (0.93 if t == 5 else 0.97), (a, ok.mean())


def test_analytic_shapes(O):
    """Sphere and torus bases without elevation equal their closed forms."""
    W = workloads()
    P = W.sphere_fbm(amp=0.0)
    p = np.random.default_rng(1).uniform(-2, 2, size=(200, 3)).astype(np.float32)
    np.testing.assert_allclose(O.synth_points(P, p), np.linalg.norm(p.astype(np.float64), axis=1) - 1.0, atol=1e-12)
    abi = W.abi
    T = abi.SynthProgram()
    T.base = abi.BASE_TORUS
    T.param[0], T.param[1] = 1.0, 0.4
    q = p.astype(np.float64)
    ref = np.hypot(np.hypot(q[:, 0], q[:, 1]) - 1.0, q[:, 2]) - 0.4
    np.testing.assert_allclose(O.synth_points(T, p), ref, atol=1e-6)


def test_smooth_union_closed_form(O):
    """smoothMin (math.cpp:28-33) of a far torus and a sphere: far apart it is
    the minimum; within k it is b + (a - b) h - k h (1 - h)."""
    W = workloads()
    abi = W.abi
    P = abi.SynthProgram()
    P.base = abi.BASE_TORUS_SPHERES
    P.param[0], P.param[1] = 2.0, 0.5
    P.n_spheres = 1
    P.sphere[0][3] = 0.5
    P.k = 0.4
    for z in (0.1, 0.9, 1.05):
        p = np.array([[0.0, 0.0, z]], np.float32)
        q = np.float64(np.float32(z))
        a = np.hypot(2.0, q) - 0.5     # torus (axis z, R = 2, r = 0.5) at (0, 0, z)
        b = q - 0.5                    # sphere r = 0.5
        h = min(max((b - a) / 0.4 * 0.5 + 0.5, 0.0), 1.0)
        expect = b + (a - b) * h - 0.4 * h * (1 - h)
        assert abs(O.synth_points(P, p)[0] - expect) < 1e-12
    p = np.array([[0.0, 0.0, 0.1]], np.float32)
    assert abs(O.synth_points(P, p)[0] - (np.float64(np.float32(0.1)) - 0.5)) < 1e-12


def test_theta_gradient_matches_finite_differences(O):
    """dd/dtheta by forward mode against FP64 central differences on the 25
    parameters of the torus/spheres/ridged/cellular planet."""
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    x = np.random.default_rng(5).uniform(-1.4, 1.4, size=(64, 3)).astype(np.float32)
    w = np.ones(len(x))
    th = O.synth_theta(P)
    g = O.synth_theta_grad(P, x, w, theta=th)
    for j in range(len(th)):
        h = 1e-6 * max(1.0, abs(th[j]))
        tp = th.copy(); tp[j] += h
        tm = th.copy(); tm[j] -= h
        fd = (O.synth_points(P, x, theta=tp).sum() - O.synth_points(P, x, theta=tm).sum()) / (2 * h)
        assert abs(fd - g[j]) <= 1e-4 * (1 + abs(g[j])), (j, fd, g[j])


def test_flop_count_constant(O):
    """The benchmark's algorithmic FLOPs per sample equal the oracle's count."""
    W = workloads()
    x = np.random.default_rng(0).uniform(-1.6, 1.6, size=(20000, 3)).astype(np.float32)
    c = O.synth_count_ops(W.torus_spheres_ridged_cellular(), x)
    assert abs(c["flop"] - W.FLOPS_PER_SAMPLE_C2) / W.FLOPS_PER_SAMPLE_C2 < 0.01
    # value with gradient, sparse forward mode over the same counting scalar
    cg = O.synth_count_ops_grad(W.torus_spheres_ridged_cellular(), x)
    assert abs(cg["flop"] - W.FLOPS_PER_SAMPLE_C2_FWD_GRAD) / W.FLOPS_PER_SAMPLE_C2_FWD_GRAD < 0.01
    assert cg["sqrt"] == c["sqrt"] and cg["floor"] == c["floor"]


def test_forward_mode_count_exceeds_value_count(O):
    """Each operation on a quantity that depends on p also updates three
    derivative lanes, so the value-with-gradient count of the plain method is
    more than three times its value count."""
    W = workloads()
    P = W.sphere_fbm()
    x = np.random.default_rng(3).uniform(-1.3, 1.3, size=(500, 3)).astype(np.float32)
    c = O.synth_count_ops_grad(P, x)
    assert c["flop"] > 3 * O.synth_count_ops(P, x)["flop"]
