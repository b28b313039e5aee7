"""Synthetic planet workloads (seeded, unit scale).

Planet programs of the benchmark configurations. Amplitudes are per octave:
a_i = amp * gain^i / sum_j gain^j (the FBM normalisation divides by the sum
of the octave gains, so `amp` is the peak displacement), frequencies
f_i = freq * lacunarity^i. All random draws use numpy's PCG64 generator
(numpy.random.default_rng), which is stable across platforms.
"""
from __future__ import annotations

import numpy as np

from . import abi


def _layer(L: abi.NoiseLayer, type_, fractal, octaves, freq, amp, seed, gain=0.5, lac=2.0, distance=0, operation=1):
    L.type = type_
    L.fractal = fractal
    L.octaves = octaves
    L.distance = distance
    L.operation = operation
    L.seed = seed
    bound = sum(abs(gain) ** i for i in range(octaves)) if fractal != abi.FRACTAL_NONE else 1.0
    for i in range(8):
        L.amp[i] = amp * gain ** i / bound if i < octaves else 0.0
        L.freq[i] = freq * lac ** i if i < octaves else 0.0


def sphere_fbm(R=1.0, octaves=4, freq=2.0, lac=2.0, gain=0.5, amp=0.05, seed=1337, noise=abi.NOISE_SIMPLEX) -> abi.SynthProgram:
    """Unit sphere minus an FBM displacement (the CPU-runnable plain method)."""
    P = abi.SynthProgram()
    P.base = abi.BASE_SPHERE
    P.param[0] = R
    P.n_layers = 1
    _layer(P.layer[0], noise, abi.FRACTAL_FBM, octaves, freq, amp, seed, gain, lac)
    return P


def torus_spheres_ridged_cellular(seed=42) -> abi.SynthProgram:
    """Torus (1.0, 0.4) smooth-unioned (k = 0.1) with 8 spheres (centres
    U[-1,1]^3, radii U[0.1,0.3]) minus 6-octave ridged Perlin (freq 3, gain 0.5,
    amp 0.04) plus a cellular F2-F1 layer (freq 8, amp 0.02; Euclidean)."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-1.0, 1.0, size=(8, 3))
    radii = rng.uniform(0.1, 0.3, size=8)
    P = abi.SynthProgram()
    P.base = abi.BASE_TORUS_SPHERES
    P.param[0] = 1.0
    P.param[1] = 0.4
    P.n_spheres = 8
    for s in range(8):
        for a in range(3):
            P.sphere[s][a] = float(centres[s, a])
        P.sphere[s][3] = float(radii[s])
    P.k = 0.1
    P.n_layers = 2
    _layer(P.layer[0], abi.NOISE_PERLIN, abi.FRACTAL_RIDGED, 6, 3.0, 0.04, seed)
    _layer(P.layer[1], abi.NOISE_CELLULAR, abi.FRACTAL_NONE, 1, 8.0, 0.02, seed + 8, distance=abi.DIST_EUCLIDEAN,
           operation=abi.OP_SUBTRACT)
    return P


def mixed_planet(rng: np.random.Generator) -> abi.SynthProgram:
    """One planet of the batched-chunk set: sphere R=1, torus (1.0, 0.4) or
    rounded cube (half-extent 0.8, rounding 0.1), 4-6 octave simplex or
    Perlin FBM (freq 2, gain 0.5, amp 0.05)."""
    P = abi.SynthProgram()
    kind = int(rng.integers(0, 3))
    if kind == 0:
        P.base = abi.BASE_SPHERE
        P.param[0] = 1.0
    elif kind == 1:
        P.base = abi.BASE_TORUS
        P.param[0] = 1.0
        P.param[1] = 0.4
    else:
        P.base = abi.BASE_ROUNDED_BOX
        P.param[0] = 0.8
        P.param[1] = 0.1
    P.n_layers = 1
    octaves = int(rng.integers(4, 7))
    noise = abi.NOISE_SIMPLEX if rng.integers(0, 2) == 0 else abi.NOISE_PERLIN
    _layer(P.layer[0], noise, abi.FRACTAL_FBM, octaves, 2.0, 0.05, int(rng.integers(0, 2 ** 31)))
    return P


# grids of the configurations
GRID_C1 = dict(lo=(-1.3, -1.3, -1.3), hi=(1.3, 1.3, 1.3), n=(128, 128, 128))
GRID_C2 = dict(lo=(-1.6, -1.6, -1.6), hi=(1.6, 1.6, 1.6), n=(512, 512, 512))


def grid(spec: dict, n=None) -> abi.Grid:
    return abi.Grid.make(spec["lo"], spec["hi"], n or spec["n"])


def theta_count(P: abi.SynthProgram) -> int:
    n = sum(2 * P.layer[l].octaves for l in range(P.n_layers))
    return n + {abi.BASE_SPHERE: 1, abi.BASE_TORUS: 2, abi.BASE_ROUNDED_BOX: 2}.get(P.base, 3 + P.n_spheres)


def theta_of(P: abi.SynthProgram) -> np.ndarray:
    """The differentiable parameter vector (layout of up_synth_program)."""
    t = []
    for l in range(P.n_layers):
        L = P.layer[l]
        t += [L.amp[i] for i in range(L.octaves)]
        t += [L.freq[i] for i in range(L.octaves)]
    if P.base == abi.BASE_SPHERE:
        t += [P.param[0]]
    elif P.base in (abi.BASE_TORUS, abi.BASE_ROUNDED_BOX):
        t += [P.param[0], P.param[1]]
    else:
        t += [P.param[0], P.param[1]] + [P.sphere[s][3] for s in range(P.n_spheres)] + [P.k]
    return np.asarray(t, dtype=np.float32)


def theta_groups(P: abi.SynthProgram) -> dict:
    """Indices of theta_of's vector by kind: octave amplitudes, octave
    frequencies and the base shape's parameters."""
    amp, freq, o = [], [], 0
    for l in range(P.n_layers):
        k = P.layer[l].octaves
        amp += list(range(o, o + k))
        freq += list(range(o + k, o + 2 * k))
        o += 2 * k
    return {"amplitudes": amp, "frequencies": freq, "shape": list(range(o, len(theta_of(P))))}


def phase_scale(P: abi.SynthProgram, theta: np.ndarray | None = None) -> np.ndarray:
    """Per-parameter unit of relative change in phase terms: f_min / f_i for
    every octave frequency f_i of theta (theta_of(P) by default; f_min the
    smallest of them), 1 for amplitudes and the base shape. A relative change
    of one unit in frequency i then moves the noise at a point by the same
    number of lattice cells for every octave (autograd.RelativeTheta)."""
    t = theta_of(P) if theta is None else np.asarray(theta, np.float32)
    s = np.ones(len(t), np.float32)
    fi = theta_groups(P)["frequencies"]
    if fi:
        fmin = float(np.min(np.abs(t[fi])))
        for i in fi:
            s[i] = fmin / abs(float(t[i])) if t[i] != 0 else 1.0
    return s


def shell_points(P_radius: float, thickness: float, n: int, seed: int) -> np.ndarray:
    """n points uniform in the spherical shell |p| in [R - t, R + t]."""
    rng = np.random.default_rng(seed)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r0, r1 = P_radius - thickness, P_radius + thickness
    r = np.cbrt(rng.uniform(r0 ** 3, r1 ** 3, size=n))
    return (d * r[:, None]).astype(np.float32)


# Algorithmic FP32 operations per sample of torus_spheres_ridged_cellular(),
# value path, counted by the oracle's operation-counting scalar over 20000
# uniform samples of GRID_C2's box (add/sub/mul/min/max/abs/select = 1, so an
# FMA counts 2; besides these, 8 divisions, 37 square roots and 21 floors per
# sample are counted apart and not included). Checked by tests/test_oracle.py.
FLOPS_PER_SAMPLE_C2 = 960.8
# The same program's value together with its gradient dd/dp, counted with the
# oracle's sparse forward-mode scalar over the same samples (each operation on
# a quantity that depends on p also updates its three derivative lanes):
# 4434.4 FP32 operations per sample (53 divisions, 37 square roots, 21 floors
# besides). Forward mode is an upper bound on the gradient's work: the GPU
# kernel's closed-form derivatives (per-face coefficients, the cellular
# winners' difference vectors) need far fewer. Checked by tests/test_oracle.py.
FLOPS_PER_SAMPLE_C2_FWD_GRAD = 4434.4


def quad_atlas(pos: np.ndarray, nrm: np.ndarray, idx: np.ndarray, width: int, height: int):
    """Test/benchmark stand-in for the reference's meshUnwrap (which stays on
    the CPU): every dual-contouring quad (two consecutive triangles sharing a
    diagonal) gets its own square chart in a regular grid of the atlas, with
    half a texel of margin. Returns (positions, normals, uvs, indices) with
    four vertices per quad."""
    tri = idx.reshape(-1, 6).astype(np.int64)
    q = len(tri)
    a, b = tri[:, :3], tri[:, 3:]
    # diagonal = the two vertices the triangles share; v1/v3 = the others
    in_b = (a[:, :, None] == b[:, None, :]).any(axis=2)          # (q, 3) which of a's vertices are in b
    in_a = (b[:, :, None] == a[:, None, :]).any(axis=2)
    v1 = a[np.arange(q), np.argmin(in_b, axis=1)]
    v3 = b[np.arange(q), np.argmin(in_a, axis=1)]
    diag = np.where(in_b, a, -1)
    v0 = diag.max(axis=1)
    v2 = np.where(diag == v0[:, None], -1, diag).max(axis=1)
    corners = np.stack([v0, v1, v2, v3], axis=1)                  # (q, 4)
    cells = int(np.ceil(np.sqrt(q))) if q else 1
    s = min(width, height) // cells
    if s < 2:
        raise ValueError("atlas too small for one chart of at least 2x2 texels per quad")
    tx, ty = np.arange(q) % cells, np.arange(q) // cells
    cu = np.array([0.0, 1.0, 1.0, 0.0])
    cv = np.array([0.0, 0.0, 1.0, 1.0])
    u = (tx[:, None] * s + 0.5 + cu[None, :] * (s - 1.0)) / width
    v = (ty[:, None] * s + 0.5 + cv[None, :] * (s - 1.0)) / height
    P = pos[corners.reshape(-1)].astype(np.float32)
    N = nrm[corners.reshape(-1)].astype(np.float32)
    UV = np.stack([u.reshape(-1), v.reshape(-1)], axis=1).astype(np.float32)
    base = 4 * np.arange(q, dtype=np.uint32)[:, None]
    I = (base + np.array([0, 1, 2, 0, 2, 3], np.uint32)[None, :]).reshape(-1).astype(np.uint32)
    return P, N, UV, I


def chunk_set(n_planets=64, n_chunks=512, seed=7, edge_lo=16, edge_hi=192):
    """Batched-chunk workload: n_planets mixed planets (mixed_planet) and
    n_chunks chunks whose per-axis sample counts are log-uniform in
    [edge_lo, edge_hi]; every chunk box has the grid spacing 2.6/191 and is
    centred near a random point of the unit sphere (so most chunks cut the
    surface). Returns (planets list, list of (planet index, Grid))."""
    rng = np.random.default_rng(seed)
    planets = [mixed_planet(rng) for _ in range(n_planets)]
    h = 2.6 / 191.0
    chunks = []
    for _ in range(n_chunks):
        p = int(rng.integers(0, n_planets))
        n = np.exp(rng.uniform(np.log(edge_lo), np.log(edge_hi), size=3)).astype(int)
        d = rng.normal(size=3)
        centre = d / np.linalg.norm(d) * rng.uniform(0.8, 1.1)
        lo = centre - 0.5 * (n - 1) * h
        hi = lo + (n - 1) * h
        chunks.append((p, abi.Grid.make(lo.tolist(), hi.tolist(), n.tolist())))
    return planets, chunks
