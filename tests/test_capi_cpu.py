"""The C ABI on the CPU: the library loads, exports every declared symbol,
and its host-side parameter rules agree with the oracle. No kernel runs."""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import abi
from computer_graphics_lab_00_gb300 import workloads as W

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = []
    for header in sorted((ROOT / "include").glob("*.h")):
        text = header.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(sph_\w+)\s*\(", text, flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ["sph_create", "sph_destroy", "sph_step", "sph_substep", "sph_upload", "sph_download",
                     "sph_emit", "sph_grid_download", "sph_stats_compute", "sph_derive_params", "sph_fluid_substeps"]:
        assert required in names


def test_library_exports_every_declared_symbol(native):
    missing = [name for name in declared_functions() if not hasattr(native, name)]
    assert not missing, f"declared in include/*.h but not exported: {missing}"


def test_abi_version_and_struct_sizes(native):
    assert native.sph_abi_version() == abi.SPH_ABI_VERSION
    assert ctypes.sizeof(abi.SphParams) == 1856
    assert native.sph_status_string(abi.SPH_ERR_NONFINITE) == b"non-finite input"


@pytest.mark.parametrize("n", [0, 1, 511, 512, 513, 8192, 16384, 32768, 40000, 1 << 20])
def test_cell_count_rules(native, n):
    assert native.sph_cell_count_for(n) == W.cell_count_for(n)
    assert native.sph_cell_count_uncapped(n) == W.cell_count_uncapped(n)


def test_cell_count_reference_values(native):
    # gfx::cellCountFor (src/gfx/fluid.cpp:50-52) and fluid_test.cpp:193.
    assert native.sph_cell_count_for(100) == 1024
    assert native.sph_cell_count_for(16384) == 32768
    assert native.sph_cell_count_for(1 << 20) == 65536
    assert native.sph_cell_count_uncapped(1 << 20) == 1 << 21


@pytest.mark.parametrize("dt", [0.0, -1.0, 1e-4, 1 / 1200, 1 / 600, 1 / 240, 1 / 60, 1 / 30, 0.1, 100.0])
@pytest.mark.parametrize("stiffness", [1.0, 50.0, 1e5])
def test_fluid_substeps_matches_oracle(native, oracle, dt, stiffness):
    from computer_graphics_lab_00_gb300.fluid import fluid_substeps

    params = W.dam_break_16k().params
    params.stiffness = stiffness
    assert fluid_substeps(params, dt) == oracle.fluid_substeps(params, dt)


def test_derive_params_matches_oracle(native, oracle):
    from computer_graphics_lab_00_gb300.fluid import derive_fluid_params

    s = abi.SphFluidSettings()
    for a, v in enumerate((0.16, 0.32, 0.16)):
        s.emitter_half_extents[a] = v
    s.particle_radius, s.smoothing_radius, s.rest_density = 0.01, 0.04, 1000.0
    s.stiffness, s.viscosity = 50.0, 0.5
    for a in range(3):
        s.container_min[a], s.container_max[a] = 0.0, 1.0
    s.gravity[1] = -9.81
    world = W.translation((0.5, 0.5, 0.5))
    got = derive_fluid_params(s, world, 16384, 32768)
    want = oracle.derive_params(s, np.array(world, np.float32), 16384, 32768)
    assert bytes(got) == bytes(want)


def test_create_without_gpu_is_a_status_not_a_crash(native):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present; the GPU tests cover creation")
    ctx = ctypes.c_void_p()
    params = W.dam_break_16k().params
    status = native.sph_create(ctypes.byref(params), 16, 0, ctypes.byref(ctx))
    assert status == abi.SPH_ERR_NO_DEVICE
    assert not ctx.value
    bad = params.copy()
    bad.lattice[3] = 1000
    assert native.sph_create(ctypes.byref(bad), 16, 0, ctypes.byref(ctx)) == abi.SPH_ERR_INVALID_ARGUMENT
    assert native.sph_create(ctypes.byref(params), 0, 0, ctypes.byref(ctx)) == abi.SPH_ERR_INVALID_ARGUMENT
    assert native.sph_step(None, ctypes.c_float(0.01)) == abi.SPH_ERR_INVALID_ARGUMENT
