"""GB300 planet SDF -> contour -> texel path (host side).

Python view of the C ABI in include/up_abi.h: a `Planet` wraps one context.
The arrays may be numpy (host) or torch CUDA tensors (device); the library
stages host buffers itself. Every call goes to libup_gb300.so; when the
library is missing or no GPU is present the calls raise -- there is no CPU
path in the product.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi, workloads  # noqa: F401
from .abi import load


class UpError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


def _addr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        assert a.is_contiguous()
        return a.data_ptr()
    raise TypeError(type(a))


class Planet:
    """One planet context: reference modes by name, or a synthetic program."""

    def __init__(self, shape=None, elevation=None, coloring="default", poles=False, flowers=False, seed=0, program=None):
        self.lib = load()
        h = C.c_void_p()
        if program is not None:
            self.program = program
            st = self.lib.up_context_create_synthetic(C.byref(program), C.byref(h))
        else:
            self.program = None
            m = abi.Modes(shape.encode(), elevation.encode(), coloring.encode(), int(bool(poles)), int(bool(flowers)))
            st = self.lib.up_context_create(C.byref(m), C.byref(abi.Seeds(seed)), C.byref(h))
        if st != abi.UP_OK:
            raise UpError(st, self.lib.up_status_string(st).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.up_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != abi.UP_OK:
            raise UpError(st, self.lib.up_last_error(self.h).decode() or self.lib.up_status_string(st).decode())

    @property
    def shape_name(self) -> str:
        b = C.create_string_buffer(64)
        self._check(self.lib.up_context_shape_name(self.h, b, 64))
        return b.value.decode()

    @property
    def double_sided(self) -> bool:
        return bool(self.lib.up_context_double_sided(self.h))

    def set_stream(self, stream_handle: int):
        self._check(self.lib.up_context_set_stream(self.h, C.c_void_p(stream_handle)))

    def set_theta(self, theta):
        self._check(self.lib.up_context_set_theta(self.h, _addr(theta), int(theta.shape[0]) if hasattr(theta, "shape") else len(theta)))

    # ---- SDF
    def sdf_points(self, xyz, d=None, grad=None, field=abi.FIELD_LAND, want_grad=False):
        n = int(xyz.shape[0])
        if d is None:
            d = np.empty(n, np.float32)
        if want_grad and grad is None:
            grad = np.empty((n, 3), np.float32)
        self._check(self.lib.up_sdf_eval_points(self.h, field, _addr(xyz), n, _addr(d), _addr(grad)))
        return (d, grad) if want_grad else d

    def sdf_grid(self, grid: abi.Grid, fields_mask=1, outs=None, grad=None):
        n = grid.count
        if outs is None:
            outs = [np.empty(n, np.float32) if (fields_mask >> f) & 1 else None for f in range(3)]
        arr = (C.c_void_p * 3)(*[_addr(o) for o in outs])
        self._check(self.lib.up_sdf_grid(self.h, fields_mask, C.byref(grid), arr, _addr(grad)))
        return outs

    def contour(self, grid: abi.Grid, field=abi.FIELD_LAND, values=None, normals=True):
        """Returns (positions (V,3), normals (V,3) or None, indices (I,)) as numpy."""
        m = abi.MeshOut()
        st = self.lib.up_contour(self.h, field, C.byref(grid), _addr(values), C.byref(m))
        if st != abi.UP_ERR_CAPACITY:
            self._check(st)
        V, I = int(m.vertex_count), int(m.index_count)
        pos = np.empty((V, 3), np.float32)
        nrm = np.empty((V, 3), np.float32) if normals else None
        idx = np.empty(I, np.uint32)
        m = abi.MeshOut(pos.ctypes.data, nrm.ctypes.data if normals else None, idx.ctypes.data, V, I, 0, 0)
        self._check(self.lib.up_contour(self.h, field, C.byref(grid), _addr(values), C.byref(m)))
        return pos, nrm, idx

    def mesh_generate_base(self, grid: abi.Grid, field=abi.FIELD_LAND, values=None, normals=True):
        """up_mesh_generate_base: contour, largest component, water filter.
        Returns (positions (V,3), normals (V,3) or None, indices (I,)) as numpy."""
        m = abi.MeshOut()
        st = self.lib.up_mesh_generate_base(self.h, field, C.byref(grid), _addr(values), C.byref(m))
        if st != abi.UP_ERR_CAPACITY:
            self._check(st)
        V, I = int(m.vertex_count), int(m.index_count)
        pos = np.empty((V, 3), np.float32)
        nrm = np.empty((V, 3), np.float32) if normals else None
        idx = np.empty(I, np.uint32)
        m = abi.MeshOut(pos.ctypes.data, nrm.ctypes.data if normals else None, idx.ctypes.data, V, I, 0, 0)
        self._check(self.lib.up_mesh_generate_base(self.h, field, C.byref(grid), _addr(values), C.byref(m)))
        return pos, nrm, idx

    def special_to_gltf_pbr(self, special):
        """(H, W, 2) uint8 special image -> (H, W, 3) uint8 glTF metallicRoughness."""
        h, w = int(special.shape[0]), int(special.shape[1])
        out = np.empty((h, w, 3), np.uint8)
        self._check(self.lib.up_image_special_to_gltf_pbr(self.h, _addr(special), w, h, _addr(out)))
        return out

    def height_to_normal(self, height, strength=1.0):
        """(H, W) uint8 height map -> (H, W, 3) uint8 normal map."""
        h, w = int(height.shape[0]), int(height.shape[1])
        out = np.empty((h, w, 3), np.uint8)
        self._check(self.lib.up_image_height_to_normal(self.h, _addr(height), w, h, float(strength), _addr(out)))
        return out

    def param_backward(self, xyz, dL_dd, dtheta=None):
        n = int(xyz.shape[0])
        nt = int(self.lib.up_synth_theta_count(C.byref(self.program)))
        if dtheta is None:
            dtheta = np.empty(nt, np.float32)
        self._check(self.lib.up_sdf_param_backward(self.h, _addr(xyz), n, _addr(dL_dd), _addr(dtheta)))
        return dtheta

    # ---- texels
    def texture(self, purpose, pos, nrm, uv, idx, width, height, dilation=7, floats=False):
        """Texel images of an unwrapped mesh (numpy host buffers or torch
        device tensors). Returns a dict of numpy arrays: albedo (H, W, 3|4),
        special (H, W, 2), height (H, W) as uint8, and the float images when
        floats=True."""
        ach = 4 if purpose == abi.PURPOSE_WATER else 3
        n = width * height
        res = dict(albedo=np.empty((height, width, ach), np.uint8), special=np.empty((height, width, 2), np.uint8),
                   height=np.empty((height, width), np.uint8))
        if floats:
            res.update(albedo_f=np.empty((height, width, ach), np.float32), special_f=np.empty((height, width, 2), np.float32),
                       height_f=np.empty((height, width), np.float32))
        m = abi.MeshIn(_addr(pos), _addr(nrm), _addr(uv), _addr(idx), int(pos.shape[0]), int(idx.shape[0]))
        o = abi.TextureOut(_addr(res["albedo"]), _addr(res["special"]), _addr(res["height"]), _addr(res.get("albedo_f")),
                           _addr(res.get("special_f")), _addr(res.get("height_f")))
        self._check(self.lib.up_texture(self.h, purpose, C.byref(m), width, height, dilation, C.byref(o)))
        del n
        return res

    def tiles(self, purpose, pos, nrm):
        """terrainTile for n points: (floats (n, 11): albedo rgb, roughness,
        metallic, height, opacity, elevation, slope, temperature,
        precipitation; uint8 (n, 2): biome, type)."""
        n = int(pos.shape[0])
        f = {k: np.empty(n, np.float32) for k in ("roughness", "metallic", "height", "opacity", "elevation", "slope", "temperature",
                                                    "precipitation")}
        alb = np.empty((n, 3), np.float32)
        bio = np.empty(n, np.uint8)
        typ = np.empty(n, np.uint8)
        o = abi.TileOut(_addr(alb), _addr(f["roughness"]), _addr(f["metallic"]), _addr(f["height"]), _addr(f["opacity"]),
                        _addr(f["elevation"]), _addr(f["slope"]), _addr(f["temperature"]), _addr(f["precipitation"]), _addr(bio),
                        _addr(typ))
        self._check(self.lib.up_tiles(self.h, purpose, _addr(pos), _addr(nrm), n, C.byref(o)))
        out = np.concatenate([alb, np.stack([f[k] for k in ("roughness", "metallic", "height", "opacity", "elevation", "slope",
                                                            "temperature", "precipitation")], axis=1)], axis=1)
        return out, np.stack([bio, typ], axis=1)


def batch_run(planet_or_lib, planets, chunks, values=False, device=False):
    """Sample and contour many chunks (up_batch_run). `planet_or_lib` is any
    Planet (its context runs the batch). Returns dict with positions (V,3),
    indices (I,), per-chunk vertex/index offsets (n+1,) and optionally the
    concatenated sampled values."""
    ctx = planet_or_lib
    P = (abi.SynthProgram * len(planets))(*planets)
    Cs = (abi.Chunk * len(chunks))(*[abi.Chunk(p, g) for p, g in chunks])
    vo = np.zeros(len(chunks) + 1, np.uint64)
    io = np.zeros(len(chunks) + 1, np.uint64)
    nval = sum(g.count for _, g in chunks)
    if device:
        import torch
        val = torch.empty(nval, device="cuda") if values else None
    else:
        val = np.empty(nval, np.float32) if values else None
    # the sizing call already names the values buffer: the library plans exact
    # sampling when values are read and narrow-band sampling otherwise
    o = abi.BatchOut(None, None, 0, 0, vo.ctypes.data, io.ctypes.data, 0, 0, _addr(val), nval if values else 0)
    st = ctx.lib.up_batch_run(ctx.h, P, len(planets), Cs, len(chunks), C.byref(o))
    if st != abi.UP_ERR_CAPACITY:
        ctx._check(st)
    V, I = int(o.vertex_count), int(o.index_count)
    if device:
        pos = torch.empty((V, 3), device="cuda")
        idx = torch.empty(I, dtype=torch.int32, device="cuda")
    else:
        pos = np.empty((V, 3), np.float32)
        idx = np.empty(I, np.uint32)
    o = abi.BatchOut(_addr(pos), _addr(idx), V, I, vo.ctypes.data, io.ctypes.data, 0, 0, _addr(val), nval if values else 0)
    ctx._check(ctx.lib.up_batch_run(ctx.h, P, len(planets), Cs, len(chunks), C.byref(o)))
    # `o` holds raw addresses of vo/io and of the outputs: they stay referenced
    # from _args so that batch_replay writes into live memory
    return dict(positions=pos, indices=idx, vertex_offsets=vo.copy(), index_offsets=io.copy(), values=val,
                _args=(P, Cs, o, vo, io, pos, idx, val))


def batch_replay(ctx, prepared):
    """Run the same batch again (graph replay inside the library), into the
    output buffers of `prepared`."""
    P, Cs, o = prepared["_args"][:3]
    ctx._check(ctx.lib.up_batch_run(ctx.h, P, len(P), Cs, len(Cs), C.byref(o)))
