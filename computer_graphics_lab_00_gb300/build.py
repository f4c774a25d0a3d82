"""Builds the native library libsph_gb300.so in-tree, for sm_103a only.

`python -m computer_graphics_lab_00_gb300.build [--force] [--verbose]`

Each .cu under csrc/ compiles to its own object in parallel with
`-gencode arch=compute_103a,code=sm_103a`; the exact-arithmetic kernels
(grid, density, integrate) build with --fmad=false so that no multiply-add
is fused, and the host side with -ffp-contract=off for the same reason.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
CSRC = PACKAGE_DIR / "csrc"
NATIVE = PACKAGE_DIR / "_native"
OBJ = NATIVE / "obj"
LIBRARY = NATIVE / "libsph_gb300.so"
INCLUDE = PACKAGE_DIR.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", f"-I{INCLUDE}"]

# Sources whose float arithmetic must round like the reference's CPU solver.
EXACT_SOURCES = {"sph_grid.cu", "sph_forces.cu", "sph_engine.cu", "sph_capi.cu", "sph_static_grid.cu",
                 "sph_surface.cu"}


def nvcc() -> str:
    found = shutil.which("nvcc")
    if found:
        return found
    candidate = Path("/usr/local/cuda/bin/nvcc")
    if candidate.exists():
        return str(candidate)
    raise RuntimeError("nvcc not found")


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, verbose: bool, ptxas_info: bool) -> Path:
    obj = OBJ / (src.stem + ".o")
    flags = list(COMMON)
    if src.name in EXACT_SOURCES:
        flags += ["--fmad=false"]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    cmd = [nvcc(), *ARCH, *flags, "-c", str(src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), flush=True)
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{proc.stdout}\n{proc.stderr}")
    if ptxas_info or verbose:
        sys.stdout.write(proc.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = _headers()
    todo = [s for s in sources if force or ptxas_info or _stale(OBJ / (s.stem + ".o"), [s, *headers])]
    if todo:
        workers = min(len(todo), max(1, os.cpu_count() or 1))
        with ThreadPoolExecutor(max_workers=workers) as pool:
            list(pool.map(lambda s: _compile(s, verbose, ptxas_info), todo))
    objects = [OBJ / (s.stem + ".o") for s in sources]
    if force or todo or _stale(LIBRARY, objects):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(LIBRARY), *map(str, objects), "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"link failed:\n{proc.stdout}\n{proc.stderr}")
    return LIBRARY


def main() -> None:
    parser = argparse.ArgumentParser(description=__doc__)
    parser.add_argument("--force", action="store_true")
    parser.add_argument("--verbose", action="store_true")
    parser.add_argument("--ptxas-info", action="store_true", help="print registers/spills per kernel")
    args = parser.parse_args()
    print(build(force=args.force, verbose=args.verbose, ptxas_info=args.ptxas_info))


if __name__ == "__main__":
    main()
