"""ctypes wrapper of the oracle library (TEST INFRASTRUCTURE, parity unpinned).

Only the test suite, the smoke check and the CPU-baseline leg of the
benchmark use this module. It restates the reference's arithmetic on the
CPU (FP64, per-operation FP32, forward-mode dual numbers) to check the CUDA
path; it is never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIBS = {}


def _pkg_abi():
    import importlib
    root = str(HERE.parent)
    if root not in sys.path:
        sys.path.insert(0, root)
    return importlib.import_module("unnatural-planets_gb300.abi")


def lib(fast: bool = False) -> C.CDLL:
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name in _LIBS:
        return _LIBS[name]
    from . import build_oracle  # noqa: F401  (package-relative when imported as oracle.oracle)
    build_oracle.build()
    L = C.CDLL(str(HERE / "_build" / name))
    abi = _pkg_abi()
    P = C.POINTER(abi.SynthProgram)
    G = C.POINTER(abi.Grid)
    vp = C.c_void_p
    sigs = {
        "orc_mix32": (C.c_uint32, [C.c_uint32]),
        "orc_lattice_hash": (C.c_uint32, [C.c_int32, C.c_int32, C.c_int32, C.c_uint32]),
        "orc_seed_key": (C.c_uint32, [C.c_uint32]),
        "orc_noise": (None, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_uint32, vp,
                             C.c_uint64, C.c_int, vp, vp]),
        "orc_synth_theta_count": (C.c_uint64, [P]),
        "orc_synth_theta": (None, [P, vp]),
        "orc_synth_points": (None, [P, vp, vp, C.c_uint64, C.c_int, vp, vp, C.c_int]),
        "orc_synth_theta_grad": (C.c_int, [P, vp, vp, C.c_uint64, vp, vp, C.c_int]),
        "orc_synth_count_ops": (None, [P, vp, C.c_uint64, vp]),
        "orc_synth_count_ops_grad": (None, [P, vp, C.c_uint64, vp]),
        "orc_synth_grid_fp32": (None, [P, G, C.c_uint32, C.c_uint32, vp, C.c_int]),
        "orc_synth_grid_fp32_cd": (None, [P, G, C.c_uint32, C.c_uint32, C.c_float, vp, vp, C.c_int]),
        "orc_grid_positions": (None, [G, vp]),
        "orc_grid_positions_at": (None, [G, vp, C.c_uint64, vp]),
        "orc_contour_synth": (vp, [P, G, vp]),
        "orc_mesh_counts": (None, [vp, vp]),
        "orc_mesh_copy": (None, [vp, vp, vp, vp, vp, vp]),
        "orc_mesh_free": (None, [vp]),
        "orc_planet_create": (vp, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_uint32, C.c_char_p, C.c_int]),
        "orc_planet_free": (None, [vp]),
        "orc_planet_shape": (C.c_int, [vp]),
        "orc_field_points": (None, [vp, C.c_int, vp, C.c_uint64, C.c_int, vp, vp, C.c_int]),
        "orc_contour_planet": (vp, [vp, C.c_int, G, vp]),
        "orc_tiles": (None, [vp, C.c_int, vp, vp, C.c_uint64, vp, vp, C.c_int]),
        "orc_texture": (None, [vp, C.POINTER(abi.SynthProgram), C.c_int, vp, vp, vp, vp, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int,
                               vp, vp, vp, vp, vp, vp, vp, C.c_int]),
        "orc_mesh_filter": (None, [C.c_uint32, C.c_uint32, vp, vp, vp, vp]),
    }
    for n, (res, args) in sigs.items():
        f = getattr(L, n)
        f.restype = res
        f.argtypes = args
    _LIBS[name] = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data


def noise(cfg: dict, xyz: np.ndarray, precision: int = 0, grad: bool = False):
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = xyz.shape[0]
    out = np.empty(n, np.float64)
    g = np.empty((n, 3), np.float64) if grad else None
    lib().orc_noise(cfg.get("type", 3), cfg.get("fractal", 0), cfg.get("octaves", 3), cfg.get("distance", 0),
                    cfg.get("operation", 1), cfg.get("frequency", 1.0), cfg.get("lacunarity", 2.0), cfg.get("gain", 0.5),
                    cfg.get("seed", 0), _p(xyz), n, precision, _p(out), _p(g))
    return (out, g) if grad else out


def synth_points(P, xyz, theta=None, precision=0, grad=False, threads=8):
    xyz = np.ascontiguousarray(xyz, np.float32)
    n = xyz.shape[0]
    out = np.empty(n, np.float64)
    g = np.empty((n, 3), np.float64) if grad else None
    th = None if theta is None else np.ascontiguousarray(theta, np.float64)
    lib().orc_synth_points(C.byref(P), _p(th), _p(xyz), n, precision, _p(out), _p(g), threads)
    return (out, g) if grad else out


def synth_theta(P) -> np.ndarray:
    n = lib().orc_synth_theta_count(C.byref(P))
    out = np.empty(n, np.float64)
    lib().orc_synth_theta(C.byref(P), _p(out))
    return out


def synth_theta_grad(P, xyz, w, theta=None, threads=8) -> np.ndarray:
    xyz = np.ascontiguousarray(xyz, np.float32)
    w = np.ascontiguousarray(w, np.float64)
    n = lib().orc_synth_theta_count(C.byref(P))
    out = np.empty(n, np.float64)
    th = None if theta is None else np.ascontiguousarray(theta, np.float64)
    if lib().orc_synth_theta_grad(C.byref(P), _p(th), _p(xyz), xyz.shape[0], _p(w), _p(out), threads) != 0:
        raise ValueError("too many parameters")
    return out


def synth_count_ops(P, xyz) -> dict:
    xyz = np.ascontiguousarray(xyz, np.float32)
    c = np.zeros(5, np.float64)
    lib().orc_synth_count_ops(C.byref(P), _p(xyz), xyz.shape[0], _p(c))
    return dict(flop=c[0], div=c[1], sqrt=c[2], floor=c[3], transcendental=c[4])


def synth_count_ops_grad(P, xyz) -> dict:
    """operation counts per sample of the value with its gradient dd/dp
    (sparse forward mode), same bins as synth_count_ops"""
    xyz = np.ascontiguousarray(xyz, np.float32)
    c = np.zeros(5, np.float64)
    lib().orc_synth_count_ops_grad(C.byref(P), _p(xyz), xyz.shape[0], _p(c))
    return dict(flop=c[0], div=c[1], sqrt=c[2], floor=c[3], transcendental=c[4])


def synth_grid_fp32(P, grid, z0, z1, threads, fast=True) -> np.ndarray:
    nx, ny = int(grid.n[0]), int(grid.n[1])
    out = np.empty(nx * ny * (z1 - z0), np.float32)
    lib(fast).orc_synth_grid_fp32(C.byref(P), C.byref(grid), z0, z1, _p(out), threads)
    return out


def synth_grid_fp32_cd(P, grid, z0, z1, h, threads, fast=True):
    nx, ny = int(grid.n[0]), int(grid.n[1])
    n = nx * ny * (z1 - z0)
    out = np.empty(n, np.float32)
    g = np.empty(3 * n, np.float32)
    lib(fast).orc_synth_grid_fp32_cd(C.byref(P), C.byref(grid), z0, z1, h, _p(out), _p(g), threads)
    return out, g


def grid_positions(grid) -> np.ndarray:
    out = np.empty((grid.count, 3), np.float32)
    lib().orc_grid_positions(C.byref(grid), _p(out))
    return out


def grid_positions_at(grid, idx: np.ndarray) -> np.ndarray:
    """positions of the samples with linear (x-fastest) indices idx"""
    idx = np.ascontiguousarray(idx, np.uint64)
    out = np.empty((idx.shape[0], 3), np.float32)
    lib().orc_grid_positions_at(C.byref(grid), _p(idx), idx.shape[0], _p(out))
    return out


def contour_synth(P, grid, values: np.ndarray) -> dict:
    values = np.ascontiguousarray(values, np.float32)
    return _mesh(lib().orc_contour_synth(C.byref(P), C.byref(grid), _p(values)))


class Planet:
    """Oracle planet of the reference modes (shape, elevation, coloring names)."""

    def __init__(self, shape, elevation, coloring="default", poles=False, flowers=False, seed=0):
        err = C.create_string_buffer(256)
        self.h = lib().orc_planet_create(shape.encode(), elevation.encode(), coloring.encode(), int(poles), int(flowers), seed, err, 256)
        if not self.h:
            raise ValueError(err.value.decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_planet_free(self.h)
            self.h = None

    @property
    def shape_index(self) -> int:
        return lib().orc_planet_shape(self.h)

    def field(self, field, xyz, precision=0, grad=False, threads=8):
        xyz = np.ascontiguousarray(xyz, np.float32)
        n = xyz.shape[0]
        out = np.empty(n, np.float64)
        g = np.empty((n, 3), np.float64) if grad else None
        lib().orc_field_points(self.h, field, _p(xyz), n, precision, _p(out), _p(g), threads)
        return (out, g) if grad else out

    def contour(self, field, grid, values):
        values = np.ascontiguousarray(values, np.float32)
        return _mesh(lib().orc_contour_planet(self.h, field, C.byref(grid), _p(values)))

    def tiles(self, purpose, pos, nrm, threads=8):
        pos = np.ascontiguousarray(pos, np.float32)
        nrm = np.ascontiguousarray(nrm, np.float32)
        n = pos.shape[0]
        out = np.empty((n, 11), np.float64)
        bt = np.empty((n, 2), np.int32)
        lib().orc_tiles(self.h, purpose, _p(pos), _p(nrm), n, _p(out), _p(bt), threads)
        return out, bt


def _mesh(h) -> dict:
    try:
        c = np.zeros(4, np.uint64)
        lib().orc_mesh_counts(h, _p(c))
        V, I, E = int(c[0]), int(c[1]), int(c[2])
        r = dict(cells=np.empty(V, np.uint64), positions=np.empty((V, 3), np.float32), normals=np.empty((V, 3), np.float32),
                 indices=np.empty(I, np.uint32), edges=np.empty(E, np.uint64))
        lib().orc_mesh_copy(h, _p(r["cells"]), _p(r["positions"]), _p(r["normals"]), _p(r["indices"]), _p(r["edges"]))
        return r
    finally:
        lib().orc_mesh_free(h)


def texture(purpose, pos, nrm, uv, idx, W, H, dilation=7, planet=None, program=None, threads=8) -> dict:
    """Texel images of a mesh: float images (NaN where uncovered), 8-bit images
    and the owning triangle per texel (-1 uncovered)."""
    pos, nrm = np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(nrm, np.float32)
    uv, idx = np.ascontiguousarray(uv, np.float32), np.ascontiguousarray(idx, np.uint32)
    ach = 4 if purpose == 2 else 3
    r = dict(albedo_f=np.empty((H, W, ach), np.float32), special_f=np.empty((H, W, 2), np.float32), height_f=np.empty((H, W), np.float32),
             albedo=np.empty((H, W, ach), np.uint8), special=np.empty((H, W, 2), np.uint8), height=np.empty((H, W), np.uint8),
             owner=np.empty((H, W), np.int32))
    lib().orc_texture(planet.h if planet is not None else None, C.byref(program) if program is not None else None, purpose, _p(pos),
                      _p(nrm), _p(uv), _p(idx), idx.shape[0], W, H, dilation, _p(r["albedo_f"]), _p(r["special_f"]),
                      _p(r["height_f"]), _p(r["albedo"]), _p(r["special"]), _p(r["height"]), _p(r["owner"]), threads)
    return r


def mesh_filter(pos, nrm, idx, valid=None):
    """meshGenerateBase* hygiene on a contoured mesh (orc_mesh_filter):
    largest component, and for water (valid = per-vertex elevationRaw < 0.1)
    the two-ring filter; then ordered compaction. Returns (pos, nrm, idx)."""
    idx = np.ascontiguousarray(idx, np.uint32)
    V, T = int(pos.shape[0]), int(idx.shape[0]) // 3
    keep_v = np.zeros(V, np.uint8)
    keep_t = np.zeros(T, np.uint8)
    va = None if valid is None else np.ascontiguousarray(valid, np.uint8)
    lib().orc_mesh_filter(V, T, _p(idx), _p(va), _p(keep_v), _p(keep_t))
    kv, kt = keep_v.astype(bool), keep_t.astype(bool)
    newidx = np.cumsum(kv) - 1
    tri = idx.reshape(-1, 3)[kt]
    return pos[kv], (None if nrm is None else nrm[kv]), newidx[tri].reshape(-1).astype(np.uint32)


def special_to_gltf_pbr(special: np.ndarray) -> np.ndarray:
    """imageConvertSpecialToGltfPbr, project definition: (255, roughness, metallic)."""
    h, w = special.shape[:2]
    out = np.empty((h, w, 3), np.uint8)
    out[..., 0] = 255
    out[..., 1:] = special
    return out


def height_to_normal(height: np.ndarray, strength: float = 1.0) -> np.ndarray:
    """imageConvertHeigthToNormal, project definition: h = height/255,
    n = normalize(-s dh/dx, -s dh/dy, 1), central differences in texels,
    one-sided at the border; (n + 1)/2 * 255 rounded. FP64."""
    h = height.astype(np.float64)
    dx = np.zeros_like(h)
    dy = np.zeros_like(h)
    if h.shape[1] > 1:
        dx[:, 1:-1] = 0.5 * (h[:, 2:] - h[:, :-2])
        dx[:, 0] = h[:, 1] - h[:, 0]
        dx[:, -1] = h[:, -1] - h[:, -2]
    if h.shape[0] > 1:
        dy[1:-1, :] = 0.5 * (h[2:, :] - h[:-2, :])
        dy[0, :] = h[1, :] - h[0, :]
        dy[-1, :] = h[-1, :] - h[-2, :]
    n = np.stack([-strength * dx / 255.0, -strength * dy / 255.0, np.ones_like(h)], axis=-1)
    n /= np.linalg.norm(n, axis=-1, keepdims=True)
    return np.floor(np.clip(n * 0.5 + 0.5, 0, 1) * 255 + 0.5).astype(np.uint8)
