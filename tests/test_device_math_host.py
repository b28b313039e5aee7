"""The CUDA path's device arithmetic headers (csrc/*.cuh), compiled as host
C++ by tests/hostcheck, against the FP64 oracle: every noise type with its
analytic gradient, both synthetic programs, and the parameter adjoint. This
checks arithmetic without a GPU; the kernels are checked in the gpu tests."""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import abi as _abi, workloads

sys.path.insert(0, str(Path(__file__).parent / "hostcheck"))
import build_hostcheck  # noqa: E402


@pytest.fixture(scope="module")
def H():
    L = C.CDLL(str(build_hostcheck.build()))
    abi = _abi()
    vp = C.c_void_p
    L.hc_noise.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, vp, C.c_uint64, vp, vp]
    L.hc_synth.argtypes = [C.POINTER(abi.SynthProgram), vp, C.c_uint64, vp, vp]
    L.hc_synth_bwd.argtypes = [C.POINTER(abi.SynthProgram), vp, C.c_uint64, vp, vp]
    L.hc_synth_bwd.restype = C.c_int
    L.hc_lattice_hash.restype = C.c_uint32
    L.hc_lattice_hash.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32]
    L.hc_corner_hash.restype = C.c_uint32
    L.hc_corner_hash.argtypes = [C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_int]
    L.hc_grid_runs.argtypes = [C.POINTER(abi.SynthProgram), vp, vp, vp, vp, vp]
    L.hc_noise_bound.restype = C.c_float
    L.hc_noise_bound.argtypes = [C.c_int, C.c_int, C.c_int]
    L.hc_synth_noise_bound.restype = C.c_float
    L.hc_synth_noise_bound.argtypes = [C.POINTER(abi.SynthProgram)]
    return L


def test_hash_bit_exact(H, O):
    r = np.random.default_rng(0)
    L = O.lib()
    for x, y, z, k in r.integers(-2 ** 31, 2 ** 31 - 2, size=(2000, 4)):
        k = int(k) & 0xFFFFFFFF
        h = L.orc_lattice_hash(int(x), int(y), int(z), k)
        assert H.hc_lattice_hash(int(x), int(y), int(z), k) == h
        # the shared-product corner form equals the direct hash for all 8 corners
        for b in range(8):
            assert H.hc_corner_hash(int(x), int(y), int(z), k, b) == L.orc_lattice_hash(
                int(x) + (b & 1), int(y) + ((b >> 1) & 1), int(z) + (b >> 2), k)


CASES = [(t, 0, 1) for t in range(5)] + [(5, d, op) for d in range(3) for op in range(7)]


@pytest.mark.parametrize("t,dist,op", CASES)
def test_noise_value_and_gradient(H, O, t, dist, op):
    x = np.random.default_rng(t * 31 + dist * 7 + op).uniform(-20, 20, size=(5000, 3)).astype(np.float32)
    key = O.lib().orc_seed_key(11)
    out = np.empty(len(x), np.float32)
    g = np.empty((len(x), 3), np.float32)
    H.hc_noise(t, dist, op, key, x.ctypes.data, len(x), out.ctypes.data, g.ctypes.data)
    ref, rg = O.noise(dict(type=t, seed=11, distance=dist, operation=op), x, grad=True)
    # FP32 evaluation of coordinates up to |20|: position rounding ~1e-6
    assert np.abs(out - ref).max() < 5e-5
    assert np.abs(g - rg).max() < 5e-4 * (1 + np.abs(rg).max())


@pytest.mark.parametrize("which", ["c1", "c2"])
def test_synth_value_gradient_adjoint(H, O, which):
    W = workloads()
    P = W.sphere_fbm() if which == "c1" else W.torus_spheres_ridged_cellular()
    xs = np.random.default_rng(2).uniform(-1.5, 1.5, size=(5000, 3)).astype(np.float32)
    out = np.empty(len(xs), np.float32)
    g = np.empty((len(xs), 3), np.float32)
    H.hc_synth(C.byref(P), xs.ctypes.data, len(xs), out.ctypes.data, g.ctypes.data)
    ref, rg = O.synth_points(P, xs, grad=True)
    assert np.abs(out - ref).max() < 1e-5
    assert np.abs(g - rg).max() < 1e-4
    w = np.random.default_rng(3).normal(size=len(xs)).astype(np.float32)
    dt = np.zeros(64)
    m = H.hc_synth_bwd(C.byref(P), xs.ctypes.data, len(xs), w.ctypes.data, dt.ctypes.data)
    rt = O.synth_theta_grad(P, xs, w.astype(np.float64))
    assert m == len(rt)
    np.testing.assert_allclose(dt[:m], rt, rtol=1e-4, atol=1e-3)


@pytest.mark.parametrize("n", [(48, 40, 36), (61, 33, 20)])
def test_grid_runs_equal_per_sample(H, O, n):
    """The x-coherent grid path (up_grid_runs.cuh) against the per-sample
    evaluation and the FP64 oracle on the Perlin + cellular program, with
    ragged run tails (61 is not a multiple of the run length)."""
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    g = W.grid(W.GRID_C2, n=n)
    lo = np.array(g.lo[:], np.float32)
    st = np.array([(g.hi[a] - g.lo[a]) / np.float32(g.n[a] - 1) for a in range(3)], np.float32)
    nn = np.array(n, np.uint32)
    N = g.count
    out = np.empty(N, np.float32)
    gr = np.empty(3 * N, np.float32)
    H.hc_grid_runs(C.byref(P), lo.ctypes.data, st.ctypes.data, nn.ctypes.data, out.ctypes.data, gr.ctypes.data)
    pos = O.grid_positions(g)
    ps = np.empty(N, np.float32)
    pg = np.empty((N, 3), np.float32)
    H.hc_synth(C.byref(P), pos.ctypes.data, N, ps.ctypes.data, pg.ctypes.data)
    ref = O.synth_points(P, pos)
    assert np.abs(out - ps).max() < 2e-6
    assert np.abs(out - ref).max() < 1e-5
    # gradients agree except where a cellular F1/F2 tie flips under reassociation
    e = np.abs(gr.reshape(3, -1).T - pg).max(axis=1)
    assert (e > 1e-4).mean() <= 1e-3
    plain = np.empty(N, np.float32)
    H.hc_grid_runs(C.byref(P), lo.ctypes.data, st.ctypes.data, nn.ctypes.data, plain.ctypes.data, None)
    assert np.array_equal(plain, out)


@pytest.mark.parametrize("t,dist,op", CASES)
def test_noise_bound_holds(H, O, t, dist, op):
    """The |n| bounds behind the narrow band of contouring (noise_abs_bound)
    hold for the oracle's noise on many points, and are not vacuous."""
    x = np.random.default_rng(100 + t * 31 + dist * 7 + op).uniform(-50, 50, size=(200000, 3))
    v = O.noise(dict(type=t, seed=3, distance=dist, operation=op), x)
    b = H.hc_noise_bound(t, dist, op)
    assert np.abs(v).max() <= b
    assert np.abs(v).max() >= 0.1 * b


def test_synth_noise_bound(H, O):
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    # ridged Perlin: |1 - 2|n|| <= 2 * 1.1 - 1 per unit amplitude; cellular F2 - F1 - 1 <= sqrt(6) - 1
    want = 0.04 * 1.2 + 0.02 * (6 ** 0.5 - 1)
    assert abs(H.hc_synth_noise_bound(C.byref(P)) - want) <= 1e-6


@pytest.mark.parametrize("elevation", ["none", "simple", "legacy", "lakes", "islands", "craters"])
def test_elevation_range_holds(H, O, elevation):
    """The elevation ranges behind the narrow band of reference-mode
    contouring (elevation_range) contain the oracle's raw elevation."""
    H.hc_modes_create.restype = C.c_void_p
    H.hc_modes_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_uint32]
    H.hc_elevation_range.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    H.hc_modes_free.argtypes = [C.c_void_p]
    for seed in (1, 9):
        d = H.hc_modes_create(b"sphere", elevation.encode(), b"default", 0, 0, seed)
        lo, hi = C.c_double(), C.c_double()
        H.hc_elevation_range(d, C.byref(lo), C.byref(hi))
        H.hc_modes_free(d)
        planet = O.Planet("sphere", elevation, "default", seed=seed)
        x = np.random.default_rng(seed).uniform(-2500, 2500, size=(60000, 3)).astype(np.float32)
        e = planet.field(4, x)
        assert lo.value <= e.min() and e.max() <= hi.value, (e.min(), e.max(), lo.value, hi.value)
        assert hi.value - lo.value <= 20 * max(1.0, e.max() - e.min())  # not vacuous


@pytest.mark.parametrize("elevation,shape", [("lakes", "sphere"), ("islands", "torus"), ("legacy", "box")])
def test_modes_grid_runs_equal_per_sample(H, O, elevation, shape):
    """The x-coherent reference-mode grid path (run tables of the lattice
    instances, up_modes_runs.cuh) against the per-sample fields and the FP32
    oracle, with a ragged run tail (45 is not a multiple of the run length)."""
    H.hc_modes_create.restype = C.c_void_p
    H.hc_modes_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_uint32]
    H.hc_modes_free.argtypes = [C.c_void_p]
    H.hc_modes_field.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]
    H.hc_modes_grid_runs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    d = H.hc_modes_create(shape.encode(), elevation.encode(), b"default", 0, 0, 4)
    n = (45, 30, 28)
    g = _abi().Grid.make((-2000, -1900, -1800), (2000, 1900, 1800), n)
    lo = np.array(g.lo[:], np.float32)
    st = np.array([(g.hi[a] - g.lo[a]) / np.float32(g.n[a] - 1) for a in range(3)], np.float32)
    nn = np.array(n, np.uint32)
    N = g.count
    outs = [np.empty(N, np.float32) for _ in range(3)]
    assert H.hc_modes_grid_runs(d, lo.ctypes.data, st.ctypes.data, nn.ctypes.data, 0.0, *[o.ctypes.data for o in outs]) == 1
    pos = O.grid_positions(g)
    planet = O.Planet(shape, elevation, "default", seed=4)
    for f in range(3):
        ps = np.empty(N, np.float32)
        H.hc_modes_field(d, f, pos.ctypes.data, N, ps.ctypes.data, None)
        rel = np.abs(outs[f].astype(np.float64) - ps) / np.maximum(1.0, np.abs(ps))
        assert (rel > 1e-5).mean() <= 1e-3, (f, rel.max())
        ref = planet.field(f, pos, precision=1)
        assert (np.abs(outs[f].astype(np.float64) - ref) / np.maximum(1.0, np.abs(ref)) > 1e-4).mean() <= 5e-3
    H.hc_modes_free(d)


def test_segment_sphere_culling_is_exact(H):
    """synth_segment_spheres: a sphere left out of a run's mask would be
    skipped by synth_base's own test at every sample, so the union (value and
    gradient) is bit-identical with and without the mask; the mask does drop
    spheres (the runs kernel's saving is real)."""
    W = workloads()
    H.hc_segment_base.restype = C.c_uint32
    H.hc_segment_base.argtypes = [C.POINTER(_abi().SynthProgram), C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_void_p, C.c_void_p]
    P = W.torus_spheres_ridged_cellular()
    r = np.random.default_rng(5)
    R = 16
    dropped = 0
    for t in range(4000):
        if t % 2:  # segments through or next to a sphere
            s = int(r.integers(P.n_spheres))
            c = np.array(P.sphere[s][:3]) + r.normal(0, P.sphere[s][3] + P.k, 3)
        else:
            c = r.uniform(-1.6, 1.6, 3)
        ln = float(r.uniform(0.0, 0.2))
        x0, y, z = np.float32(c[0] - ln / 2), np.float32(c[1]), np.float32(c[2])
        x1 = np.float32(x0 + ln)
        om = np.empty(4 * R, np.float32)
        of = np.empty(4 * R, np.float32)
        live = H.hc_segment_base(C.byref(P), x0, x1, y, z, R, om.ctypes.data, of.ctypes.data)
        assert np.array_equal(om, of), (x0, x1, y, z, live)
        dropped += P.n_spheres - bin(live & ((1 << P.n_spheres) - 1)).count("1")
    assert dropped > 4000 * P.n_spheres // 2


def test_fastdiv_exact(H):
    """The multiply-shift division by a fixed divisor (up_fastdiv.h, used for
    the chunk dimensions of batches) equals integer division for divisors
    1 .. 4096, powers of two and large values, on edge and random dividends."""
    H.hc_fastdiv.argtypes = [C.c_uint32, C.c_void_p, C.c_uint64, C.c_void_p]
    r = np.random.default_rng(8)
    divisors = list(range(1, 4097)) + [2 ** k for k in range(32)] + [2 ** k + 1 for k in range(1, 31)] + [2 ** 32 - 1, 2 ** 31 - 1]
    divisors += [int(x) for x in r.integers(1, 2 ** 32, size=200)]
    for d in divisors:
        n = np.concatenate([np.array([0, 1, d - 1, d, d + 1, 2 ** 32 - 1, 2 ** 32 - 2], dtype=np.uint64) % 2 ** 32,
                            r.integers(0, 2 ** 32, size=64, dtype=np.uint64)]).astype(np.uint32)
        q = np.empty_like(n)
        H.hc_fastdiv(d, n.ctypes.data, len(n), q.ctypes.data)
        assert np.array_equal(q, n // np.uint32(d)), d


def test_row_sign_bits_unaligned(H):
    """Sign words written per 16-sample row segment (the narrow-band grid
    kernels, x extents not a multiple of 16: bits OR-ed into zeroed words)
    equal the words packed from the per-sample signs, for ragged rows whose
    segments straddle word boundaries; the padding words stay zero."""
    H.hc_row_signs.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
    r = np.random.default_rng(21)
    for nx in (17, 31, 33, 45, 100, 131, 200):
        nrows = 37
        npts = nx * nrows
        neg = r.random(npts) < 0.5
        neg[r.integers(0, npts, size=npts // 4)] = False
        p0, m = [], []
        for row in range(nrows):
            for i0 in range(0, nx, 16):
                ln = min(16, nx - i0)
                bits = neg[row * nx + i0: row * nx + i0 + ln]
                p0.append(row * nx + i0)
                m.append(int(np.sum(bits.astype(np.uint64) << np.arange(ln, dtype=np.uint64))))
        p0 = np.array(p0, dtype=np.uint64)
        m = np.array(m, dtype=np.uint32)
        nwords = (npts + 31) // 32 + 2
        words = np.zeros(nwords, dtype=np.uint32)
        H.hc_row_signs(p0.ctypes.data, m.ctypes.data, len(p0), words.ctypes.data)
        padded = np.zeros(nwords * 32, dtype=bool)
        padded[:npts] = neg
        want = np.packbits(padded.reshape(-1, 8), axis=1, bitorder="little").reshape(-1).view("<u4")
        assert np.array_equal(words, want), nx


@pytest.mark.parametrize("k", range(4))
def test_task_band_classification(H, O, k):
    """The task-level narrow band (synth_task_band_kernel's test, compiled for
    the host): every sample of a task classified outside the band has
    |base| > band and the sign of the task's value, and so has the oracle's
    exact SDF there (the layers stay below the band); most tasks of the
    benchmark planet are outside. Ragged grids: x, y, z extents not multiples
    of the task's 16 x 8 x 4."""
    H.hc_task_band.restype = C.c_float
    H.hc_task_band.argtypes = [C.POINTER(_abi().SynthProgram), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    H.hc_base_grid.argtypes = [C.POINTER(_abi().SynthProgram), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    W = workloads()
    rng = np.random.default_rng(5)
    cases = [(W.torus_spheres_ridged_cellular(), (131, 117, 103), 0.6), (W.torus_spheres_ridged_cellular(), (64, 56, 48), 0.0),
             (W.mixed_planet(rng), (70, 41, 37), 0.3), (W.mixed_planet(rng), (96, 64, 60), 0.3)]
    P, n, min_far = cases[k]
    lo = np.full(3, -1.6, np.float32)
    nn = np.array(n, np.uint32)
    step = (np.float32(3.2) / (nn - 1).astype(np.float32)).astype(np.float32)
    nt = (-(-n[0] // 16)) * (-(-n[1] // 8)) * (-(-n[2] // 4))
    tv = np.empty(nt, np.float32)
    band = H.hc_task_band(C.byref(P), lo.ctypes.data, step.ctypes.data, nn.ctypes.data, tv.ctypes.data)
    base = np.empty(n[0] * n[1] * n[2], np.float32)
    H.hc_base_grid(C.byref(P), lo.ctypes.data, step.ctypes.data, nn.ctypes.data, base.ctypes.data)
    base = base.reshape(n[2], n[1], n[0])
    kk, jj, ii = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    t = ii // 16 + (-(-n[0] // 16)) * (jj // 8 + (-(-n[1] // 8)) * (kk // 4))
    far = ~np.isnan(tv)
    assert far.mean() >= min_far
    fs = far[t]
    assert np.all(np.abs(base[fs]) > band)
    assert np.all(np.sign(base[fs]) == np.sign(tv[t][fs]))
    if k == 1:  # the exact SDF keeps the sign on a small grid
        x = [lo[a] + np.arange(n[a], dtype=np.float32) * step[a] for a in range(3)]
        zz, yy, xx = np.meshgrid(x[2], x[1], x[0], indexing="ij")
        pts = np.stack([xx, yy, zz], -1).reshape(-1, 3)[fs.reshape(-1)]
        d = O.synth_points(P, pts)
        assert np.all(np.sign(d) == np.sign(tv[t][fs]))


def test_narrow_band_runs_keep_signs(H, O):
    """The narrow-band runs of contouring (synth_run with a band, compiled for
    the host; there a run is one task): every sample keeps the sign of the
    exactly sampled grid; the samples whose base lies inside the band keep
    their exact values; the rest (runs filled from their midpoint, or whose
    layers were skipped) lie outside the band. Many runs are filled."""
    H.hc_grid_runs_band.argtypes = [C.POINTER(_abi().SynthProgram), C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
    W = workloads()
    P = W.torus_spheres_ridged_cellular()
    n = (96, 64, 56)
    g = W.grid(W.GRID_C2, n=n)
    lo = np.array(g.lo[:], np.float32)
    st = np.array([(g.hi[a] - g.lo[a]) / np.float32(g.n[a] - 1) for a in range(3)], np.float32)
    nn = np.array(n, np.uint32)
    band = np.float32((H.hc_synth_noise_bound(C.byref(P)) + st.max()) * 1.001 + 1e-5)
    full = np.empty(g.count, np.float32)
    H.hc_grid_runs(C.byref(P), lo.ctypes.data, st.ctypes.data, nn.ctypes.data, full.ctypes.data, None)
    banded = np.empty(g.count, np.float32)
    H.hc_grid_runs_band(C.byref(P), lo.ctypes.data, st.ctypes.data, nn.ctypes.data, band, banded.ctypes.data)
    assert np.array_equal(banded < 0, full < 0)
    # base values: the program without its layers
    P0 = W.torus_spheres_ridged_cellular()
    P0.n_layers = 0
    base = np.empty(g.count, np.float32)
    H.hc_grid_runs(C.byref(P0), lo.ctypes.data, st.ctypes.data, nn.ctypes.data, base.ctypes.data, None)
    inside = np.abs(base) <= band
    assert inside.any() and np.array_equal(banded[inside], full[inside])
    changed = banded != full
    assert changed.mean() > 0.5 and np.all(np.abs(base[changed]) > band)
    # filled runs: 16 equal values where the base varies along the run
    rows = banded.reshape(-1, n[0])[:, :96].reshape(-1, 6, 16)
    assert (np.ptp(rows, axis=2) == 0).mean() > 0.5


def test_modes_narrow_band_runs_keep_signs(H, O):
    """The reference-mode narrow band over runs (modes_run_shape, host form of
    the x-coherent kernel): land keeps the exact grid's signs, the samples of
    shape inside the band keep their exact values, and runs are filled."""
    H.hc_modes_create.restype = C.c_void_p
    H.hc_modes_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_uint32]
    H.hc_modes_free.argtypes = [C.c_void_p]
    H.hc_modes_band.restype = C.c_float
    H.hc_modes_band.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    H.hc_modes_grid_runs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    d = H.hc_modes_create(b"sphere", b"lakes", b"default", 0, 0, 4)
    n = (96, 50, 40)
    g = _abi().Grid.make((-2000, -2000, -2000), (2000, 2000, 2000), n)
    lo = np.array(g.lo[:], np.float32)
    st = np.array([(g.hi[a] - g.lo[a]) / np.float32(g.n[a] - 1) for a in range(3)], np.float32)
    nn = np.array(n, np.uint32)
    band = H.hc_modes_band(d, 0, st.ctypes.data)
    assert band > 0
    N = g.count
    full = [np.empty(N, np.float32) for _ in range(3)]
    banded = [np.empty(N, np.float32) for _ in range(3)]
    assert H.hc_modes_grid_runs(d, lo.ctypes.data, st.ctypes.data, nn.ctypes.data, 0.0, *[o.ctypes.data for o in full]) == 1
    assert H.hc_modes_grid_runs(d, lo.ctypes.data, st.ctypes.data, nn.ctypes.data, band, *[o.ctypes.data for o in banded]) == 1
    assert np.array_equal(banded[0] < 0, full[0] < 0)
    shape = full[1]  # water = the shape
    inside = np.abs(shape) <= band
    assert inside.any() and np.array_equal(banded[0][inside], full[0][inside])
    rows = banded[0].reshape(-1, n[0]).reshape(-1, 6, 16)
    assert (np.ptp(rows, axis=2) == 0).mean() > 0.3
    H.hc_modes_free(d)


@pytest.mark.parametrize("shape,elevation,seed,n", [("sphere", "lakes", 4, (96, 50, 40)), ("torus", "islands", 2, (70, 41, 37)),
                                                    ("box", "legacy", 3, (57, 64, 45))])
def test_modes_task_band_classification(H, shape, elevation, seed, n):
    """The reference-mode task-level band (modes_task_band_kernel's test,
    compiled for the host): every sample of a task classified outside the
    band has |shape| > band, and its land and navigation values have the
    sign of the task's value; many tasks are outside. Ragged grids."""
    H.hc_modes_create.restype = C.c_void_p
    H.hc_modes_create.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_uint32]
    H.hc_modes_free.argtypes = [C.c_void_p]
    H.hc_modes_band.restype = C.c_float
    H.hc_modes_band.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    H.hc_modes_grid_runs.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    H.hc_modes_task_band.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_void_p]
    d = H.hc_modes_create(shape.encode(), elevation.encode(), b"default", 0, 0, seed)
    g = _abi().Grid.make((-2000, -2000, -2000), (2000, 2000, 2000), n)
    lo = np.array(g.lo[:], np.float32)
    st = np.array([(g.hi[a] - g.lo[a]) / np.float32(g.n[a] - 1) for a in range(3)], np.float32)
    nn = np.array(n, np.uint32)
    full = [np.empty(g.count, np.float32) for _ in range(3)]
    assert H.hc_modes_grid_runs(d, lo.ctypes.data, st.ctypes.data, nn.ctypes.data, 0.0, *[o.ctypes.data for o in full]) == 1
    nt = (-(-n[0] // 16)) * (-(-n[1] // 8)) * (-(-n[2] // 4))
    kk, jj, ii = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    t = (ii // 16 + (-(-n[0] // 16)) * (jj // 8 + (-(-n[1] // 8)) * (kk // 4))).reshape(-1)
    for field in (0, 2):  # land, navigation
        band = H.hc_modes_band(d, field, st.ctypes.data)
        assert band > 0
        tv = np.empty(nt, np.float32)
        H.hc_modes_task_band(d, lo.ctypes.data, st.ctypes.data, nn.ctypes.data, band, tv.ctypes.data)
        far = ~np.isnan(tv)
        assert far.mean() > 0.2
        fs = far[t]
        assert np.all(np.abs(full[1][fs]) > band)  # water = the shape
        assert np.all(np.sign(full[field][fs]) == np.sign(tv[t][fs]))
    H.hc_modes_free(d)



def test_pointer_placement_rule(H):
    """The C ABI uses a caller's buffer in place only when it is device memory
    of the context's GPU or managed memory; host memory and memory of another
    GPU are staged through the context's scratch (a kernel never makes a peer
    access). Arguments: query ok, cudaMemoryType, attribute device, context device."""
    H.hc_ptr_kind.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int]
    H.hc_ptr_kind.restype = C.c_int
    HOST, LOCAL, OTHER = 0, 1, 2
    assert H.hc_ptr_kind(1, 2, 0, 0) == LOCAL      # device memory of this GPU
    assert H.hc_ptr_kind(1, 2, 3, 3) == LOCAL
    assert H.hc_ptr_kind(1, 2, 1, 0) == OTHER      # device memory of another GPU
    assert H.hc_ptr_kind(1, 2, 0, 1) == OTHER
    assert H.hc_ptr_kind(1, 3, 5, 0) == LOCAL      # managed memory, any device
    assert H.hc_ptr_kind(1, 1, 0, 0) == HOST       # page-locked host memory
    assert H.hc_ptr_kind(1, 0, -2, 0) == HOST      # unregistered host memory
    assert H.hc_ptr_kind(0, 2, 0, 0) == HOST       # the query failed: treated as host memory


@pytest.mark.parametrize("spread,lane_spread", [(0.35, 0.35), (0.9, 0.15), (1.0, 1.0)])
def test_cellular_pruning_keeps_both_keys(H, spread, lane_spread):
    """The warp-wide pruning of the cellular table (cell_box_bounds,
    cell_entry_everywhere, cell_entry_in_some_window, cell_prune_bound of
    up_grid_runs.cuh) never drops one of a sample's two nearest candidates:
    over random warps, sub-runs and tables, every lane and sample keeps the
    two keys of the unpruned search. The realistic case (a 512^3 sub-run
    spans about 0.35 x 0.35 x 0.15 cells) keeps a small share of the entries."""
    H.hc_prune_check.restype = C.c_int
    H.hc_prune_check.argtypes = [C.c_uint32, C.c_int, C.c_double, C.c_double, C.c_void_p, C.c_void_p]
    kept, total = C.c_uint64(0), C.c_uint64(0)
    bad = H.hc_prune_check(11, 3000, spread, lane_spread, C.byref(kept), C.byref(total))
    assert bad == 0
    assert 0 < kept.value < total.value
    if (spread, lane_spread) == (0.35, 0.35):
        assert kept.value / total.value < 0.35


def test_mix32_split_equals_mix32(H):
    """mix32(a ^ b) == mix32_tail(mix32_head(a) ^ mix32_head(b)): the first
    mixing step (x ^= x >> 16) distributes over xor, which lets the lattice
    runs form the y/z half once per run and the x half once per face."""
    H.hc_mix32_split.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
    r = np.random.default_rng(4)
    a = r.integers(0, 2 ** 32, size=1 << 16, dtype=np.uint64).astype(np.uint32)
    b = r.integers(0, 2 ** 32, size=1 << 16, dtype=np.uint64).astype(np.uint32)
    a[:4] = [0, 0xFFFFFFFF, 0x8000, 0x10000]
    b[:4] = [0, 0xFFFFFFFF, 0x8000, 0xFFFF]
    out = np.zeros(len(a), np.uint8)
    H.hc_mix32_split(a.ctypes.data, b.ctypes.data, len(a), out.ctypes.data)
    assert out.all()


def test_ridged_sign_flip_equals_select(H):
    """The lattice runs' ridged derivative factor by a sign-bit flip equals
    the select form bit for bit, zero at n = +-0 included."""
    H.hc_ridged_sign.argtypes = [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p]
    r = np.random.default_rng(5)
    k2 = (r.standard_normal(1 << 16) * 0.1).astype(np.float32)
    nv = r.standard_normal(1 << 16).astype(np.float32)
    nv[:6] = [0.0, -0.0, 1e-45, -1e-45, np.inf, -np.inf]
    k2[:6] = [0.08, -0.08, 0.08, 0.08, -0.5, 0.5]
    out = np.zeros(len(nv), np.uint8)
    H.hc_ridged_sign(k2.ctypes.data, nv.ctypes.data, len(nv), out.ctypes.data)
    assert out.all()
