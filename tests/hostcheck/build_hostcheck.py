"""Builds tests/hostcheck/_build/libhostcheck.so (test harness only)."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def build() -> Path:
    out = HERE / "_build" / "libhostcheck.so"
    out.parent.mkdir(exist_ok=True)
    src = HERE / "device_math_host.cpp"
    csrc = HERE.parent.parent / "unnatural-planets_gb300" / "csrc"
    deps = [src, *csrc.glob("*.cuh"), *csrc.glob("*.h"), csrc / "up_modes_host.cpp", HERE.parent.parent / "include" / "up_abi.h"]
    if out.exists() and out.stat().st_mtime >= max(p.stat().st_mtime for p in deps):
        return out
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-Wno-unknown-pragmas", str(src), str(csrc / "up_modes_host.cpp"),
                        "-o", str(out)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    return out
