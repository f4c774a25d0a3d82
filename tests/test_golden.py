"""Golden vectors made by the reference itself (tests/golden/make_golden.py):
the oracle on the CPU, and the CUDA path on the GPU, must reproduce them
bit for bit. These run where the reference tree is absent."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.abi import SphParams

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name: str):
    data = dict(np.load(GOLDEN / f"{name}.npz"))
    params = SphParams.from_buffer_copy(data.pop("params").tobytes())
    return params, data


def same(a, b) -> bool:
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def compact(counts, slots):
    filled = np.minimum(counts, 32)
    used = (np.arange(32)[None, :] < filled[:, None]).reshape(-1)
    return slots[used]


def test_generators_reproduce_golden_inputs():
    params, g = load("dam_break_small")
    pos, vel = W.jittered_block(params, 2048, seed=11)
    assert same(pos, g["pos"]) and same(vel, g["vel"])
    scene, s = load("scene_frames")
    assert bytes(scene) == bytes(W.reference_test_scene(1024))
    obstacles, o = load("obstacles_small")
    assert bytes(obstacles) == bytes(W.obstacles_small())
    pos, vel = W.jittered_block(obstacles, 2048, seed=13)
    assert same(pos, o["pos"]) and same(vel, o["vel"])


def test_oracle_colliders_and_fields(oracle):
    params, g = load("obstacles_small")
    for k in (1, 40):
        pos, vel = oracle.run_substeps(params, g["pos"], g["vel"], 1.0 / 600.0, k, threads=3)
        assert same(pos, g[f"pos_{k}"]) and same(vel, g[f"vel_{k}"])


def test_oracle_scene_frames(oracle):
    params, g = load("scene_frames")
    pos, vel = oracle.emit(params, 1024)
    assert same(pos, g["emit_pos"]) and same(vel, g["emit_vel"])
    pos, vel = oracle.step(params, pos, vel, 1.0 / 60.0, threads=4, frames=30)
    assert same(pos, g["pos_30"]) and same(vel, g["vel_30"])


@pytest.mark.parametrize("name,steps", [("dam_break_small", (1, 20)), ("collisions_overflow", (5,))])
def test_oracle_grid_and_substeps(oracle, name, steps):
    params, g = load(name)
    cell_of, counts, slots = oracle.grid_build(params, g["pos"])
    np.testing.assert_array_equal(cell_of, g["cell_of"])
    np.testing.assert_array_equal(counts, g["cell_counts"])
    np.testing.assert_array_equal(compact(counts, slots), g["cell_slots"])
    for k in steps:
        pos, vel = oracle.run_substeps(params, g["pos"], g["vel"], 1.0 / 600.0, k, threads=3)
        assert same(pos, g[f"pos_{k}"]) and same(vel, g[f"vel_{k}"])


@pytest.mark.gpu
def test_gpu_matches_golden(native):
    from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

    params, g = load("scene_frames")
    with FluidSolverGpu(params, 1024) as solver:
        solver.emit(params, 1024)
        pos, vel = solver.state()
        assert same(pos, g["emit_pos"]) and same(vel, g["emit_vel"])
        for _ in range(30):
            solver.step(params, 1.0 / 60.0)
        pos, vel = solver.state()
        assert same(pos, g["pos_30"]) and same(vel, g["vel_30"])
    for name, steps in (("dam_break_small", (1, 20)), ("collisions_overflow", (5,))):
        params, g = load(name)
        with FluidSolverGpu(params, g["pos"].shape[0]) as solver:
            solver.upload(g["pos"], g["vel"])
            solver.build_grid()
            cell_of, counts, slots = solver.grid()
            np.testing.assert_array_equal(cell_of, g["cell_of"])
            np.testing.assert_array_equal(counts, g["cell_counts"])
            np.testing.assert_array_equal(compact(counts, slots), g["cell_slots"])
            done = 0
            for k in steps:
                solver.run(1.0 / 600.0, k - done)
                done = k
                pos, vel = solver.state()
                assert same(pos, g[f"pos_{k}"]) and same(vel, g[f"vel_{k}"]), f"{name} after {k}"
    params, g = load("obstacles_small")
    with FluidSolverGpu(params, 2048) as solver:
        solver.upload(g["pos"], g["vel"])
        done = 0
        for k in (1, 40):
            solver.run(1.0 / 600.0, k - done)
            done = k
            pos, vel = solver.state()
            assert same(pos, g[f"pos_{k}"]) and same(vel, g[f"vel_{k}"]), f"obstacles_small after {k}"
