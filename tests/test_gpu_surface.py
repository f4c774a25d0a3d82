"""The fluid surface on the GPU against the oracle and the golden vectors,
bit for bit: field samples by their IEEE bits, vertices by their 16 bytes
(position and packed normal) in the reference's serial order."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import abi
from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.abi import SphParams
from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu, march_field

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name):
    data = dict(np.load(GOLDEN / f"{name}.npz"))
    return SphParams.from_buffer_copy(data.pop("params").tobytes()), data


def geometry(params, resolution):
    origin = np.array(params.container_min[:3], np.float32)
    cell = ((np.array(params.container_max[:3], np.float32) - origin) / np.float32(resolution)).astype(np.float32)
    return origin, cell


def same_vertices(a, b):
    return np.array_equal(np.asarray(a).view(np.uint8).reshape(-1, 16), np.asarray(b).view(np.uint8).reshape(-1, 16))


def test_golden_surface(native):
    params, g = load("surface_small")
    with FluidSolverGpu(params, 2048) as solver:
        solver.upload(g["pos"])
        solver.surface_field(24)
        field = solver.field()
        np.testing.assert_array_equal(field.view(np.uint32), g["field_24"].view(np.uint32))
        n = solver.surface_march(0.5, 200000)
        assert same_vertices(solver.surface_vertices(n), g["vertices_24"])
        n = solver.surface_march(0.5, 600)
        assert same_vertices(solver.surface_vertices(n), g["vertices_24_cap600"])
        assert solver.surface_march(0.5, 2) == 0


@pytest.mark.parametrize("resolution", [16, 48, 128])
def test_dam_break_surface_matches_oracle(native, oracle, resolution):
    case = W.dam_break_16k()
    pos, vel = case.initial_state()
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        solver.run(case.dt, 120)
        gp, _ = solver.state()
        solver.surface_field(resolution)
        field = solver.field()
        n = solver.surface_march(0.5, 400000)
        verts = solver.surface_vertices(n)
    want = oracle.surface_field(case.params, gp, resolution, threads=16)
    np.testing.assert_array_equal(field.view(np.uint32), want.view(np.uint32))
    origin, cell = geometry(case.params, resolution)
    expect = oracle.march_field(want, resolution, origin, cell, 0.5, 400000)
    assert n == len(expect) and n > 0
    assert same_vertices(verts, expect)


def test_capacity_cut_matches_oracle(native, oracle):
    case = W.dam_break_16k()
    pos, vel = case.initial_state()
    origin, cell = geometry(case.params, 48)
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        solver.surface_field(48)
        field = solver.field()
        total = solver.surface_march(0.5, 1 << 20)
        for capacity in (3, 4, 1000, 1001, total - 1, total, total + 5):
            n = solver.surface_march(0.5, capacity)
            expect = oracle.march_field(field, 48, origin, cell, 0.5, capacity)
            assert n == len(expect) <= capacity
            assert same_vertices(solver.surface_vertices(n), expect)


@pytest.mark.parametrize("iso", [0.05, 0.5, 2.0])
def test_march_field_standalone_matches_oracle(native, oracle, iso):
    """sph_march_field on fields the solver did not make: a sphere (the
    reference test's field, with negative values) and random noise."""
    resolution = 24
    samples = resolution + 1
    idx = np.arange(samples, dtype=np.float32)
    coord = idx / np.float32(resolution) * np.float32(2.0) - np.float32(1.0)
    z, y, x = np.meshgrid(coord, coord, coord, indexing="ij")
    sphere = (np.float32(0.6) - np.sqrt(x * x + y * y + z * z)).astype(np.float32).reshape(-1)
    noise = np.random.default_rng(7).uniform(0, 3, samples ** 3).astype(np.float32)
    cell = np.float32(2.0) / np.float32(resolution)
    for field in (sphere, noise):
        got = march_field(field, resolution, (-1, -1, -1), (cell, cell, cell), iso, 300000)
        expect = oracle.march_field(field, resolution, (-1, -1, -1), (cell, cell, cell), iso, 300000)
        assert len(got) == len(expect)
        assert same_vertices(got, expect)


def test_surface_of_one_million_particles(native, oracle):
    case = W.dam_break_1m()
    pos, vel = case.initial_state()
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        solver.run(case.dt, 2)
        gp, _ = solver.state()
        solver.surface_field(128)
        field = solver.field()
        n = solver.surface_march(0.5, 2_000_000)
        verts = solver.surface_vertices(n)
    want = oracle.surface_field(case.params, gp, 128, threads=16)
    np.testing.assert_array_equal(field.view(np.uint32), want.view(np.uint32))
    origin, cell = geometry(case.params, 128)
    expect = oracle.march_field(want, 128, origin, cell, 0.5, 2_000_000)
    assert same_vertices(verts, expect)


def test_empty_and_invalid(native):
    case = W.dam_break_16k()
    with FluidSolverGpu(case.params, 16) as solver:
        with pytest.raises(abi.SphError) as e:
            solver.surface_march(0.5, 100)  # no field yet
        assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT
        solver.surface_field(8)
        assert not solver.field().any()
        assert solver.surface_march(0.5, 100) == 0
        for bad in (0, abi.SPH_SURFACE_MAX_RESOLUTION + 1):
            with pytest.raises(abi.SphError) as e:
                solver.surface_field(bad)
            assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT
