"""include/setops_gpu.hpp, the C++ face of the C ABI shaped like the
reference's visitor API: it compiles on its own (CPU), and a self-checking
program using every wrapper runs on the GPU."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "hpp_check.cpp"
PKG = ROOT / "simd_set_operations_gb300"


def test_header_compiles():
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-fsyntax-only",
                    f"-I{ROOT / 'include'}", str(SRC)], check=True)


@pytest.mark.gpu
def test_header_program_runs(tmp_path):
    exe = tmp_path / "hpp_check"
    subprocess.run(["g++", "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(SRC), "-o", str(exe),
                    f"-L{PKG}", "-lsetops_gpu", f"-Wl,-rpath,{PKG}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
