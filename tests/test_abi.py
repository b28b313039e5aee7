"""The C-ABI library loads on a CPU-only machine and exports every entry
point that include/up_abi.h declares (no compute calls without a GPU)."""
from __future__ import annotations

import ctypes as C

from conftest import abi as _abi, pkg


def test_library_exports_every_header_symbol():
    abi = _abi()
    lib = abi.load(build_if_missing=True)
    names = abi.header_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the ctypes signature table covers the header exactly
    assert sorted(n for n, _, _ in abi.SIGNATURES) == names


def test_pure_host_entry_points():
    abi = _abi()
    lib = abi.load(build_if_missing=True)
    assert lib.up_status_string(abi.UP_ERR_NAN) == b"invalid sdf value"
    assert lib.up_status_string(0) == b"ok"
    W = pkg().workloads
    assert lib.up_synth_theta_count(C.byref(W.torus_spheres_ridged_cellular())) == 25
    assert lib.up_synth_theta_count(C.byref(W.sphere_fbm())) == 9
    # instance seeds are a fixed function of (seed, slot)
    a = lib.up_instance_seed(42, 3)
    assert a == lib.up_instance_seed(42, 3) and a != lib.up_instance_seed(42, 4)


def test_struct_layout_matches_header():
    abi = _abi()
    assert C.sizeof(abi.NoiseLayer) == 6 * 4 + 16 * 4
    assert C.sizeof(abi.SynthProgram) == 4 + 8 + 4 + 128 + 4 + 4 + 2 * C.sizeof(abi.NoiseLayer)
    assert C.sizeof(abi.Grid) == 36
