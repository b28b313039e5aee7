"""ctypes view of the C ABI declared in include/up_abi.h.

The structures mirror the header field by field. Buffers are passed as raw
addresses (numpy `.ctypes.data` or torch `data_ptr()`); the library decides
host versus device from the pointer itself.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

UP_OK = 0
UP_ERR_INVALID_ARGUMENT = 1
UP_ERR_INVALID_MODE = 2
UP_ERR_NAN = 3
UP_ERR_OOM = 4
UP_ERR_CUDA = 5
UP_ERR_CAPACITY = 6
UP_ERR_TIMEOUT = 7
UP_ERR_EMPTY_MESH = 8
UP_ERR_NO_DEVICE = 9

FIELD_LAND, FIELD_WATER, FIELD_NAVIGATION, FIELD_ELEVATION, FIELD_ELEVATION_RAW = range(5)
PURPOSE_UNDEFINED, PURPOSE_LAND, PURPOSE_WATER, PURPOSE_NAVIGATION = range(4)
NOISE_VALUE, NOISE_CUBIC, NOISE_PERLIN, NOISE_SIMPLEX, NOISE_SIMPLEX_REDUCED, NOISE_CELLULAR = range(6)
FRACTAL_NONE, FRACTAL_FBM, FRACTAL_RIDGED = range(3)
DIST_EUCLIDEAN, DIST_MANHATTAN, DIST_HYBRID = range(3)
OP_CELL, OP_DISTANCE, OP_DISTANCE2, OP_ADD, OP_SUBTRACT, OP_MULTIPLY, OP_DIVIDE = range(7)
BASE_SPHERE, BASE_TORUS, BASE_ROUNDED_BOX, BASE_TORUS_SPHERES = range(4)


class NoiseLayer(C.Structure):
    _fields_ = [("type", C.c_int32), ("fractal", C.c_int32), ("octaves", C.c_int32), ("distance", C.c_int32),
                ("operation", C.c_int32), ("seed", C.c_uint32), ("amp", C.c_float * 8), ("freq", C.c_float * 8)]


class SynthProgram(C.Structure):
    _fields_ = [("base", C.c_int32), ("param", C.c_float * 2), ("n_spheres", C.c_int32), ("sphere", (C.c_float * 4) * 8),
                ("k", C.c_float), ("n_layers", C.c_int32), ("layer", NoiseLayer * 2)]


class Grid(C.Structure):
    _fields_ = [("lo", C.c_float * 3), ("hi", C.c_float * 3), ("n", C.c_uint32 * 3)]

    @staticmethod
    def make(lo, hi, n):
        g = Grid()
        for a in range(3):
            g.lo[a] = lo[a]
            g.hi[a] = hi[a]
            g.n[a] = n[a]
        return g

    @property
    def count(self) -> int:
        return int(self.n[0]) * int(self.n[1]) * int(self.n[2])


class MeshOut(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("indices", C.c_void_p), ("vertex_capacity", C.c_uint64),
                ("index_capacity", C.c_uint64), ("vertex_count", C.c_uint64), ("index_count", C.c_uint64)]


class MeshIn(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p), ("indices", C.c_void_p),
                ("vertex_count", C.c_uint64), ("index_count", C.c_uint64)]


class TextureOut(C.Structure):
    _fields_ = [("albedo", C.c_void_p), ("special", C.c_void_p), ("height", C.c_void_p), ("albedo_f32", C.c_void_p),
                ("special_f32", C.c_void_p), ("height_f32", C.c_void_p)]


class TileOut(C.Structure):
    _fields_ = [("albedo", C.c_void_p), ("roughness", C.c_void_p), ("metallic", C.c_void_p), ("height", C.c_void_p),
                ("opacity", C.c_void_p), ("elevation", C.c_void_p), ("slope", C.c_void_p), ("temperature", C.c_void_p),
                ("precipitation", C.c_void_p), ("biome", C.c_void_p), ("type", C.c_void_p)]


class Modes(C.Structure):
    _fields_ = [("shape", C.c_char_p), ("elevation", C.c_char_p), ("coloring", C.c_char_p), ("poles", C.c_int32),
                ("flowers", C.c_int32)]


class Seeds(C.Structure):
    _fields_ = [("seed", C.c_uint32)]


class Chunk(C.Structure):
    _fields_ = [("planet", C.c_uint32), ("grid", Grid)]


class BatchOut(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("indices", C.c_void_p), ("vertex_capacity", C.c_uint64),
                ("index_capacity", C.c_uint64), ("chunk_vertex_offset", C.c_void_p), ("chunk_index_offset", C.c_void_p),
                ("vertex_count", C.c_uint64), ("index_count", C.c_uint64), ("values", C.c_void_p), ("values_capacity", C.c_uint64)]


# (name, restype, argtypes) of every entry point in include/up_abi.h
SIGNATURES = [
    ("up_context_create", C.c_int, [C.POINTER(Modes), C.POINTER(Seeds), C.POINTER(C.c_void_p)]),
    ("up_context_create_synthetic", C.c_int, [C.POINTER(SynthProgram), C.POINTER(C.c_void_p)]),
    ("up_context_destroy", C.c_int, [C.c_void_p]),
    ("up_context_set_stream", C.c_int, [C.c_void_p, C.c_void_p]),
    ("up_context_shape_name", C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    ("up_context_double_sided", C.c_int, [C.c_void_p]),
    ("up_context_set_theta", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    ("up_synth_theta_count", C.c_size_t, [C.POINTER(SynthProgram)]),
    ("up_status_string", C.c_char_p, [C.c_int]),
    ("up_last_error", C.c_char_p, [C.c_void_p]),
    ("up_context_device_bytes", C.c_size_t, [C.c_void_p]),
    ("up_debug_fail_allocations", None, [C.c_uint32]),
    ("up_debug_set_wait_limit", None, [C.c_uint64]),
    ("up_debug_set_batch_form", C.c_int, [C.c_int]),
    ("up_instance_seed", C.c_uint32, [C.c_uint32, C.c_uint32]),
    ("up_sdf_eval_points", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    ("up_set_current_context", C.c_int, [C.c_void_p]),
    ("up_sdf_land", C.c_float, [C.c_void_p]),
    ("up_sdf_water", C.c_float, [C.c_void_p]),
    ("up_sdf_navigation", C.c_float, [C.c_void_p]),
    ("up_sdf_grid", C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(Grid), C.c_void_p * 3, C.c_void_p]),
    ("up_contour", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Grid), C.c_void_p, C.POINTER(MeshOut)]),
    ("up_mesh_generate_base", C.c_int, [C.c_void_p, C.c_int, C.POINTER(Grid), C.c_void_p, C.POINTER(MeshOut)]),
    ("up_image_special_to_gltf_pbr", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]),
    ("up_image_height_to_normal", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_float, C.c_void_p]),
    ("up_texture", C.c_int, [C.c_void_p, C.c_int, C.POINTER(MeshIn), C.c_uint32, C.c_uint32, C.c_int, C.POINTER(TextureOut)]),
    ("up_tiles", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(TileOut)]),
    ("up_sdf_param_backward", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    ("up_sdf_param_backward_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    ("up_batch_run", C.c_int, [C.c_void_p, C.POINTER(SynthProgram), C.c_size_t, C.POINTER(Chunk), C.c_size_t, C.POINTER(BatchOut)]),
]

_LIB = None


def library_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load libup_gb300.so. Raises if it is not built: there is no CPU fallback."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run __graft_entry__.build() (the CUDA library is required)")
        _build.build()
    lib = C.CDLL(str(path))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name, None)
        if fn is None:
            continue  # reported by the symbol-export test
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def header_symbols() -> list[str]:
    """Every function name declared in include/up_abi.h (parsed from the header)."""
    import re
    text = (Path(__file__).resolve().parent.parent / "include" / "up_abi.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(up_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))
