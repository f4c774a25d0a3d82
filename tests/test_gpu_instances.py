"""The device instance writer (fluid_instances.comp; CPU twin
src/gfx/fluid.cpp:402-466) against records built on the host from the
particle positions."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from computer_graphics_lab_00_gb300 import abi
from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

pytestmark = pytest.mark.gpu


def expected_instances(pos, prev, radius, mesh):
    n = len(pos)
    out = np.zeros(n, abi.INSTANCE)
    for key, src in (("model", pos), ("previous_model", prev)):
        m = np.zeros((n, 16), np.float32)
        m[:, 0] = m[:, 5] = m[:, 10] = radius
        m[:, 12:15] = src[:, :3]
        m[:, 15] = 1.0
        out[key] = m
    out["normal_matrix"] = np.eye(4, dtype=np.float32).reshape(16)
    out["mesh_index"] = mesh
    out["joint_offset"] = out["skinned_vertex_offset"] = out["previous_skinned_vertex_offset"] = 0xFFFFFFFF
    return out


def test_instances_and_tlas_records(native):
    params = W.reference_test_scene(1024)
    radius = np.float32(params.container_min[3])
    base, tbase = 5, 3
    with FluidSolverGpu(params, 1024) as solver:
        solver.emit(params, 1024)
        for _ in range(3):
            solver.step(params, 1.0 / 60.0)
        pos = solver.particles()
        prev = solver.previous_particles()
        assert not np.array_equal(pos, prev)
        inst = torch.zeros((base + 1024) * abi.INSTANCE.itemsize, dtype=torch.uint8, device="cuda")
        tlas = torch.zeros((tbase + 1024) * abi.TLAS_INSTANCE.itemsize, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()  # the zero fill runs on torch's stream, the writer on the solver's
        solver.write_instances(inst.data_ptr(), base, 7, tlas.data_ptr(), tbase, 0x1234_5678_9ABC, 0,
                               abi.SPH_INSTANCES_WRITE_TLAS)
        solver.synchronize()
        got = inst.cpu().numpy().view(abi.INSTANCE)
        want = expected_instances(pos, prev, radius, 7)
        assert got[:base].view(np.uint8).max() == 0
        np.testing.assert_array_equal(got[base:].view(np.uint8), want.view(np.uint8))
        t = tlas.cpu().numpy().view(abi.TLAS_INSTANCE)[tbase:]
        rows = np.zeros((1024, 12), np.float32)
        rows[:, 0] = rows[:, 5] = rows[:, 10] = radius
        rows[:, 3], rows[:, 7], rows[:, 11] = pos[:, 0], pos[:, 1], pos[:, 2]
        np.testing.assert_array_equal(t["transform"], rows)
        np.testing.assert_array_equal(t["custom_index_mask"], (np.arange(1024) + base) | (0xFF << 24))
        assert (t["blas"] == 0x1234_5678_9ABC).all() and (t["sbt_offset_flags"] == 0).all()
        # keepRendered: the previous positions are now the current ones.
        np.testing.assert_array_equal(solver.previous_particles(), pos)
        # Surface mode and a fresh emit (history reset).
        solver.write_instances(inst.data_ptr(), 0, 7, tlas.data_ptr(), 0, 0xABCD, 3,
                               abi.SPH_INSTANCES_WRITE_TLAS | abi.SPH_INSTANCES_SURFACE_TLAS
                               | abi.SPH_INSTANCES_RESET_HISTORY)
        solver.synchronize()
        got = inst.cpu().numpy().view(abi.INSTANCE)[:1024]
        np.testing.assert_array_equal(got["previous_model"], got["model"])
        t = tlas.cpu().numpy().view(abi.TLAS_INSTANCE)[:1024]
        np.testing.assert_array_equal(t["transform"][0], np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32))
        assert t["custom_index_mask"][0] == (0x800000 | 3) | (1 << 24) and t["sbt_offset_flags"][0] == 1 << 24
        assert t["blas"][0] == 0xABCD and not t[1:].view(np.uint8).any()
        with pytest.raises(abi.SphError):
            solver.write_instances(inst.data_ptr() + 4, 0, 7)


@pytest.mark.parametrize("flags", [abi.SPH_INSTANCES_WRITE_TLAS, 0, abi.SPH_INSTANCES_RESET_HISTORY,
                                   abi.SPH_INSTANCES_WRITE_TLAS | abi.SPH_INSTANCES_SURFACE_TLAS])
def test_instances_equal_the_oracle(native, oracle, flags):
    """Device records against the oracle's restatement of the reference's
    CPU writer (fluid.cpp:402-466), byte for byte, at 1M particles."""
    case = W.dam_break_1m()
    n = case.count
    radius = np.float32(case.params.container_min[3])
    with FluidSolverGpu(case.params, n) as solver:
        solver.upload(*case.initial_state())
        solver.run(case.dt, 2)
        pos = solver.particles()
        prev = solver.previous_particles()
        inst = torch.zeros((n + 3) * abi.INSTANCE.itemsize, dtype=torch.uint8, device="cuda")
        tlas = torch.zeros((n + 2) * abi.TLAS_INSTANCE.itemsize, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()  # the zero fill runs on torch's stream, the writer on the solver's
        solver.write_instances(inst.data_ptr(), 3, 5, tlas.data_ptr(), 2, 0x1234_5678_9ABC, 6, flags)
        solver.synchronize()
        got = inst.cpu().numpy().view(abi.INSTANCE)
        got_t = tlas.cpu().numpy().view(abi.TLAS_INSTANCE)
        np.testing.assert_array_equal(solver.previous_particles(), pos)  # keepRendered
    want = np.zeros(n + 3, abi.INSTANCE)
    want_t = np.zeros(n + 2, abi.TLAS_INSTANCE)
    oracle.write_instances(pos, prev, radius, want, 3, 5, want_t, 2, 0x1234_5678_9ABC, 6, flags,
                           threads=oracle.hardware_threads)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert np.array_equal(got_t.view(np.uint8), want_t.view(np.uint8))



@pytest.mark.parametrize("count", [1, 31, 33, 1000])
def test_ragged_counts_write_only_their_records(native, oracle, count):
    """Counts that leave a warp partly empty: the records equal the oracle's,
    nothing past the last record is written, and keepRendered covers every
    particle."""
    params = W.reference_test_scene(count)
    radius = np.float32(params.container_min[3])
    with FluidSolverGpu(params, count) as solver:
        solver.emit(params, count)
        for _ in range(2):
            solver.step(params, 1.0 / 60.0)
        pos = solver.particles()
        prev = solver.previous_particles()
        inst = torch.full(((count + 40) * abi.INSTANCE.itemsize,), 0xA5, dtype=torch.uint8, device="cuda")
        tlas = torch.full(((count + 40) * abi.TLAS_INSTANCE.itemsize,), 0xA5, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        solver.write_instances(inst.data_ptr(), 1, 2, tlas.data_ptr(), 4, 0x77, 0, abi.SPH_INSTANCES_WRITE_TLAS)
        solver.synchronize()
        got = inst.cpu().numpy().view(abi.INSTANCE)
        got_t = tlas.cpu().numpy().view(abi.TLAS_INSTANCE)
        np.testing.assert_array_equal(solver.previous_particles(), pos)
    want = np.zeros(count + 40, abi.INSTANCE)
    want_t = np.zeros(count + 40, abi.TLAS_INSTANCE)
    want.view(np.uint8)[:] = 0xA5
    want_t.view(np.uint8)[:] = 0xA5
    oracle.write_instances(pos, prev, radius, want, 1, 2, want_t, 4, 0x77, 0, abi.SPH_INSTANCES_WRITE_TLAS)
    assert np.array_equal(got.view(np.uint8), want.view(np.uint8))
    assert np.array_equal(got_t.view(np.uint8), want_t.view(np.uint8))
