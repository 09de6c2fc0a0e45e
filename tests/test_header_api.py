"""The drop-in C++ header (include/t1m/t1m.h): it compiles as C++20 against
the C-ABI library (CPU), and the reference-style program runs correctly on
the GPU (tests/cpp/header_api.cpp)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "header_api.cpp"
OUT = ROOT / "tests" / "_build" / "header_api"


def _compile(built_lib):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    OUT.parent.mkdir(parents=True, exist_ok=True)
    libdir = Path(built_lib).parent
    cmd = [cxx, "-std=c++20", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
           str(SRC), f"-L{libdir}", "-lt1m_cuda", f"-Wl,-rpath,{libdir}", "-o", str(OUT)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return OUT


def test_header_compiles_and_links(built_lib):
    assert _compile(built_lib).exists()


@pytest.mark.gpu
def test_header_program_runs_on_gpu(built_lib):
    exe = _compile(built_lib)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "header api ok" in r.stdout
