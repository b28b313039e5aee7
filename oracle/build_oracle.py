"""Build recipe for the oracle (test infrastructure; see oracle_core.hpp).

Produces oracle/_build/liboracle.so (FP32 restatement rounded per operation,
-ffp-contract=off, the parity checker) and oracle/_build/liboracle_fast.so
(same source with the compiler's default contraction, the timed CPU
baseline). Plain g++ invocations, no architecture-specific flags.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SRC = HERE / "oracle_capi.cpp"
LIBS = {"liboracle.so": ["-ffp-contract=off"], "liboracle_fast.so": []}


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    deps = [SRC, *HERE.glob("*.hpp"), HERE.parent / "include" / "up_abi.h"]
    newest = max(p.stat().st_mtime for p in deps)
    for name, extra in LIBS.items():
        out = BUILD / name
        if out.exists() and out.stat().st_mtime >= newest:
            continue
        cmd = [cxx, "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", *extra, str(SRC), "-o", str(out) + ".tmp"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
        os.replace(str(out) + ".tmp", out)
    return BUILD / "liboracle.so"


if __name__ == "__main__":
    print(build(verbose=True))
