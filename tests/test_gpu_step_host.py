"""sph_step_host: upload, substeps and download in one call, with the
velocity upload overlapping the first substep's grid build (and, from 2^18
particles, the density pass, with the download overlapping integrate). Same
bits as sph_upload + sph_run + sph_download, the same checks, and the
reference's substep (oracle) underneath."""
from __future__ import annotations

import numpy as np
import pytest
import torch

from computer_graphics_lab_00_gb300 import abi
from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def state_after(case, substeps):
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(*case.initial_state())
        solver.run(case.dt, substeps)
        return solver.state()


@pytest.mark.parametrize("substeps", [1, 3])
@pytest.mark.parametrize("make", [W.dam_break_16k, W.obstacle_course])
def test_equals_upload_run_download(native, make, substeps):
    case = make()
    pos, vel = state_after(case, 4)
    with FluidSolverGpu(case.params, case.count) as a, FluidSolverGpu(case.params, case.count) as b:
        a.upload(pos, vel)
        a.run(case.dt, substeps)
        want_p, want_v = a.state()
        got_p, got_v = b.step_host_arrays(pos, vel, case.dt, substeps)
        assert np.array_equal(bits(got_p), bits(want_p))
        assert np.array_equal(bits(got_v), bits(want_v))
        # The context holds the stepped state, and previous = the uploaded positions.
        p, v = b.state()
        assert np.array_equal(bits(p), bits(want_p)) and np.array_equal(bits(v), bits(want_v))
        assert np.array_equal(bits(b.previous_particles()), bits(a.previous_particles()))


def test_one_substep_equals_the_oracle(native, oracle):
    case = W.dam_break_16k()
    pos, vel = state_after(case, 2)
    want_p, want_v = oracle.run_substeps(case.params, pos.copy(), vel.copy(), case.dt, 1,
                                         threads=oracle.hardware_threads)
    with FluidSolverGpu(case.params, case.count) as s:
        got_p, got_v = s.step_host_arrays(pos, vel, case.dt, 1)
    assert np.array_equal(bits(got_p), bits(want_p)) and np.array_equal(bits(got_v), bits(want_v))


def test_pinned_in_place_at_1m_over_repeated_calls(native):
    """The end-to-end loop: pinned host arrays stepped in place call after
    call (the Morton order carried across calls) against the device-resident
    run."""
    case = W.dam_break_1m()
    pos0, vel0 = case.initial_state()
    host_p = torch.from_numpy(pos0.copy()).pin_memory()
    host_v = torch.from_numpy(vel0.copy()).pin_memory()
    with FluidSolverGpu(case.params, case.count) as a, FluidSolverGpu(case.params, case.count) as b:
        a.upload(pos0, vel0)
        a.run(case.dt, 12)
        want_p, want_v = a.state()
        for _ in range(12):
            b.step_host(host_p.data_ptr(), host_v.data_ptr(), case.count, case.dt, 1, host_p.data_ptr(),
                        host_v.data_ptr())
    assert np.array_equal(bits(host_p.numpy()), bits(want_p))
    assert np.array_equal(bits(host_v.numpy()), bits(want_v))


def test_optional_arrays(native):
    case = W.dam_break_16k()
    pos, _ = state_after(case, 3)
    with FluidSolverGpu(case.params, case.count) as a, FluidSolverGpu(case.params, case.count) as b:
        a.upload(pos, None)  # zero velocities
        a.run(case.dt, 2)
        want_p, _ = a.state()
        out_p = np.full_like(pos, 7.0)
        b.step_host(pos.ctypes.data, None, case.count, case.dt, 2, out_p.ctypes.data, None)
        assert np.array_equal(bits(out_p), bits(want_p))


def test_rejects_nonfinite_and_leaves_the_outputs(native):
    case = W.dam_break_16k()
    pos, vel = state_after(case, 2)
    for which, value in (("vel", np.nan), ("pos", np.inf)):
        p, v = pos.copy(), vel.copy()
        (v if which == "vel" else p)[1234, 1] = value
        out_p = np.full_like(pos, 3.0)
        out_v = np.full_like(pos, 5.0)
        with FluidSolverGpu(case.params, case.count) as s:
            with pytest.raises(abi.SphError) as e:
                s.step_host(p.ctypes.data, v.ctypes.data, case.count, case.dt, 2, out_p.ctypes.data,
                            out_v.ctypes.data)
            assert e.value.status == abi.SPH_ERR_NONFINITE
            assert (out_p == 3.0).all() and (out_v == 5.0).all()
            # The context stays usable: a clean call afterwards is exact.
            got_p, got_v = s.step_host_arrays(pos, vel, case.dt, 1)
        with FluidSolverGpu(case.params, case.count) as a:
            a.upload(pos, vel)
            a.run(case.dt, 1)
            want_p, want_v = a.state()
        assert np.array_equal(bits(got_p), bits(want_p)) and np.array_equal(bits(got_v), bits(want_v))


def test_edge_cases(native):
    case = W.dam_break_16k()
    pos, vel = state_after(case, 1)
    with FluidSolverGpu(case.params, case.count) as s:
        with pytest.raises(abi.SphError) as e:
            s.step_host_arrays(np.zeros((case.count + 1, 4), np.float32), None, case.dt, 1)
        assert e.value.status == abi.SPH_ERR_CAPACITY
        with pytest.raises(abi.SphError) as e:
            s.step_host_arrays(pos, vel, -1.0, 1)
        assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT
        # No substeps: upload and download only.
        p, v = s.step_host_arrays(pos, vel, case.dt, 0)
        assert np.array_equal(bits(p), bits(pos)) and np.array_equal(bits(v), bits(vel))
        # No particles.
        p, v = s.step_host_arrays(np.zeros((0, 4), np.float32), None, case.dt, 1)
        assert p.shape == (0, 4)
        # A smaller count after a larger one, then the full count again.
        p, v = s.step_host_arrays(pos[:1000], vel[:1000], case.dt, 1)
        with FluidSolverGpu(case.params, case.count) as a:
            a.upload(pos[:1000], vel[:1000])
            a.run(case.dt, 1)
            want_p, want_v = a.state()
        assert np.array_equal(bits(p), bits(want_p)) and np.array_equal(bits(v), bits(want_v))
        p, v = s.step_host_arrays(pos, vel, case.dt, 1)
        assert p.shape == pos.shape


def first_particles(count, substeps_in=3):
    """The first `count` particles of the 1M dam break a few substeps in."""
    case = W.dam_break_1m()
    with FluidSolverGpu(case.params, case.count) as s:
        s.upload(*case.initial_state())
        s.run(case.dt, substeps_in)
        pos, vel = s.state()
    return case, pos[:count].copy(), vel[:count].copy()


@pytest.mark.parametrize("count,substeps,schedule,sort", [
    (300_001, 1, 1, 2),    # an odd count: cuts on 128-slot boundaries, a ragged last range
    (300_001, 3, 2, 2),    # Hilbert order, the last of three substeps in id ranges
    (1_048_576, 2, 1, 1),  # one-kernel radix passes
    (1_048_576, 1, 1, 0),  # three kernels per radix pass
    (262_144, 1, 0, 2),    # bucket order: no id ranges, the plain form
])
def test_overlapped_form_equals_upload_run_download(native, count, substeps, schedule, sort):
    """From 2^18 particles (one tank, a curve order, the mask kernels, no
    colliders) the velocities are gathered beside the density pass and the
    last integrate runs in three id ranges, each range's rows downloading
    while the next integrates; results, the context's state and previous
    positions equal the unsplit run's, call after call."""
    case, pos, vel = first_particles(count)
    with FluidSolverGpu(case.params, case.count) as a, FluidSolverGpu(case.params, case.count) as b:
        for s in (a, b):
            s.set_tuning(schedule=schedule, sort=sort)
        a.upload(pos, vel)
        b_p, b_v = pos, vel
        for call in range(3):
            a.run(case.dt, substeps)
            want_p, want_v = a.state()
            uploaded = b_p
            b_p, b_v = b.step_host_arrays(b_p, b_v, case.dt, substeps)
            assert np.array_equal(bits(b_p), bits(want_p)), call
            assert np.array_equal(bits(b_v), bits(want_v)), call
            p, v = b.state()
            assert np.array_equal(bits(p), bits(want_p)) and np.array_equal(bits(v), bits(want_v))
            # previous = the positions this call uploaded.
            assert np.array_equal(bits(b.previous_particles()), bits(uploaded)), call


def test_overlapped_form_after_run_and_back(native):
    """Alternating step_host (an order split by id range) and run (the plain
    order) keeps the bits of a run-only context."""
    case, pos, vel = first_particles(400_000)
    with FluidSolverGpu(case.params, case.count) as a, FluidSolverGpu(case.params, case.count) as b:
        a.upload(pos, vel)
        a.run(case.dt, 9)
        want_p, want_v = a.state()
        p, v = b.step_host_arrays(pos, vel, case.dt, 2)
        b.run(case.dt, 3)
        p, v = b.state()
        p, v = b.step_host_arrays(p, v, case.dt, 1)
        b.run(case.dt, 1)
        p, v = b.state()
        p, v = b.step_host_arrays(p, v, case.dt, 2)
        assert np.array_equal(bits(p), bits(want_p)) and np.array_equal(bits(v), bits(want_v))


def test_overlapped_form_optional_arrays_and_nonfinite(native):
    case, pos, vel = first_particles(300_001)
    with FluidSolverGpu(case.params, case.count) as a, FluidSolverGpu(case.params, case.count) as b:
        a.upload(pos, None)
        a.run(case.dt, 1)
        want_p, want_v = a.state()
        out_p = np.full_like(pos, 7.0)
        b.step_host(pos.ctypes.data, None, len(pos), case.dt, 1, out_p.ctypes.data, None)
        assert np.array_equal(bits(out_p), bits(want_p))
        got_v = b.state()[1]
        assert np.array_equal(bits(got_v), bits(want_v))
        bad = vel.copy()
        bad[299_999, 2] = np.nan
        out_p[:] = 3.0
        out_v = np.full_like(pos, 5.0)
        with pytest.raises(abi.SphError) as e:
            b.step_host(pos.ctypes.data, bad.ctypes.data, len(pos), case.dt, 1, out_p.ctypes.data,
                        out_v.ctypes.data)
        assert e.value.status == abi.SPH_ERR_NONFINITE
        assert (out_p == 3.0).all() and (out_v == 5.0).all()
        a.upload(pos, vel)
        a.run(case.dt, 1)
        want_p, want_v = a.state()
        got_p, got_v = b.step_host_arrays(pos, vel, case.dt, 1)
        assert np.array_equal(bits(got_p), bits(want_p)) and np.array_equal(bits(got_v), bits(want_v))
