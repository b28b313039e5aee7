"""include/up_abi.h as the reference would use it: a C++17 program (the
binding a reference maintainer would write, made into one program, with the
terrain callbacks called from eight threads at once) and a C99 program, both compiled with the system
compilers against the header and linked to libup_gb300.so. The CPU tests
compile and link them (and the header alone as C and as C++ with warnings as
errors); the GPU test runs them."""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT, abi as _abi

HERE = Path(__file__).resolve().parent / "abi_consumer"
OUT = HERE / "_build"
INCLUDE = ROOT / "include"


def _lib_dir() -> Path:
    _abi().load(build_if_missing=True)
    return Path(_abi().library_path()).parent


def _build(src: str, lang: str) -> Path:
    OUT.mkdir(exist_ok=True)
    libdir = _lib_dir()
    exe = OUT / (Path(src).stem + ("_cpp" if lang == "c++" else "_c"))
    if lang == "c++":
        cc = [os.environ.get("CXX") or shutil.which("g++") or "g++", "-std=c++17", "-pthread"]
    else:
        cc = [os.environ.get("CC") or shutil.which("gcc") or "gcc", "-std=c99"]
    cmd = [*cc, "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(INCLUDE), str(HERE / src), "-o", str(exe), f"-L{libdir}", "-lup_gb300",
           f"-Wl,-rpath,{libdir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("lang,flags", [("c", ["-std=c89", "-pedantic"]), ("c", ["-std=c11"]), ("c++", ["-std=c++11"]),
                                        ("c++", ["-std=c++20"])])
def test_header_compiles_alone(lang, flags, tmp_path):
    src = tmp_path / ("h.c" if lang == "c" else "h.cpp")
    src.write_text('#include "up_abi.h"\nint up_probe(void) { return UP_ABI_VERSION; }\n')
    cc = (shutil.which("gcc") or "gcc") if lang == "c" else (shutil.which("g++") or "g++")
    r = subprocess.run([cc, *flags, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-I", str(INCLUDE), str(src)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr


def test_consumers_compile_and_link():
    assert _build("consumer.cpp", "c++").exists()
    assert _build("consumer.c", "c").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("src,lang", [("consumer.cpp", "c++"), ("consumer.c", "c")])
def test_consumers_run(cuda, src, lang):
    exe = _build(src, lang)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "consumer" in r.stdout
