"""The C++ wrapper (include/sph_solver.hpp) compiles against the C ABI, and
on a GPU runs the reference's own fluid test blocks (tests/cpp)."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SOURCE = ROOT / "tests" / "cpp" / "fluid_solver_gpu_test.cpp"


def build(tmp_path: Path) -> Path:
    from computer_graphics_lab_00_gb300 import abi

    lib = abi.library_path()
    if not lib.exists():
        raise RuntimeError(f"native library missing at {lib}")
    exe = tmp_path / "fluid_solver_gpu_test"
    cmd = ["g++", "-std=c++17", "-O1", "-UNDEBUG", f"-I{ROOT / 'include'}", str(SOURCE), "-o", str(exe),
           f"-L{lib.parent}", "-lsph_gb300", f"-Wl,-rpath,{lib.parent}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_wrapper_compiles_and_links(tmp_path):
    assert build(tmp_path).exists()


@pytest.mark.gpu
def test_reference_fluid_blocks_on_gpu(tmp_path):
    exe = build(tmp_path)
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert "passed" in proc.stdout
