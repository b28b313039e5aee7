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

    def param_backward(self, xyz, dL_dd, dtheta=None):
        n = int(xyz.shape[0])
        nt = int(self.lib.up_synth_theta_count(C.byref(self.program)))
        if dtheta is None:
            dtheta = np.empty(nt, np.float32)
        self._check(self.lib.up_sdf_param_backward(self.h, _addr(xyz), n, _addr(dL_dd), _addr(dtheta)))
        return dtheta
