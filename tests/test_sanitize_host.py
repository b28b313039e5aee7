"""Address and undefined-behaviour sanitizers over the host-compilable code:
the oracle, the CUDA path's device arithmetic compiled for the host, the mode
tables and the index helpers of the grid kernels (tests/hostcheck/
sanitize_main.cpp drives every entry point on small inputs). A device-side
sanitizer is not available for the kernels; this run checks the same sources
on the CPU."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

from conftest import ROOT

HERE = Path(__file__).resolve().parent / "hostcheck"


def _build() -> Path:
    out = HERE / "_build" / "sanitize_main"
    out.parent.mkdir(exist_ok=True)
    csrc = ROOT / "unnatural-planets_gb300" / "csrc"
    srcs = [HERE / "sanitize_main.cpp", ROOT / "oracle" / "oracle_capi.cpp", HERE / "device_math_host.cpp", csrc / "up_modes_host.cpp"]
    deps = srcs + list(csrc.glob("*.cuh")) + list(csrc.glob("*.h")) + list((ROOT / "oracle").glob("*.hpp")) + [ROOT / "include" / "up_abi.h"]
    if out.exists() and out.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return out
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-pthread", "-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer",
           "-Wno-unknown-pragmas", *map(str, srcs), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_sanitized_host_code():
    exe = _build()
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=0:halt_on_error=1", UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, (r.stdout + r.stderr)[-6000:]
    assert "sanitized run" in r.stdout
