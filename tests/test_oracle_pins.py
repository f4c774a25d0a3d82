"""The reference's own fluid assertions (tests/fluid_test.cpp), run on the
oracle: emit lattice, containment, settling, density band, determinism
across worker counts, parameter derivation and substep bounds."""
from __future__ import annotations

import numpy as np

from computer_graphics_lab_00_gb300 import abi
from computer_graphics_lab_00_gb300 import workloads as W


def test_emit_lattice_in_box(oracle):
    # fluid_test.cpp:53-75: half extents 0.4, 512 particles, emitter at (0, 1, 0).
    s = abi.SphFluidSettings()
    for a in range(3):
        s.emitter_half_extents[a] = 0.4
        s.container_min[a], s.container_max[a] = -1.0, 1.0
    s.container_min[1], s.container_max[1] = 0.0, 2.0
    s.particle_radius, s.smoothing_radius, s.rest_density, s.stiffness, s.viscosity = 0.025, 0.1, 1000.0, 50.0, 0.5
    s.gravity[1] = -9.81
    params = oracle.derive_params(s, np.array(W.translation((0, 1, 0)), np.float32), 512, 1024)
    pos, vel = oracle.emit(params, 512)
    half = (np.array(params.lattice[:3], np.float32) - 1) * np.float32(params.spacing) * np.float32(0.5)
    local = pos[:, :3] - np.array([0, 1, 0], np.float32)
    assert np.all(np.abs(local[:, 0]) <= half[0] + 1e-4)
    assert np.all(np.abs(local[:, 1]) <= half[1] + 1e-4)
    assert abs(pos[0, 3] - params.rest_density) < 1e-3
    assert not vel.any()


def test_particles_stay_in_container_and_settle(oracle):
    # fluid_test.cpp:77-96.
    params = W.reference_test_scene(512)
    pos, vel = oracle.emit(params, 512)
    pos, vel = oracle.step(params, pos, vel, 1.0 / 60.0, threads=4, frames=60)
    for a in range(3):
        assert np.all(pos[:, a] >= params.container_min[a] - 1e-3)
        assert np.all(pos[:, a] <= params.container_max[a] + 1e-3)
    assert pos[:, 1].max() < 0.6


def test_submerged_density_band(oracle):
    # fluid_test.cpp:98-128: narrow container, 1024 particles, 120 frames.
    f32 = np.float32
    half, r = f32(0.2), f32(0.025)
    spacing = r * f32(2)
    n_axis = int(np.floor(half * f32(2) / spacing))
    params = W.make_params(container_min=(-0.25, 0.0, -0.25), container_max=(0.25, 1.0, 0.25),
                           lattice=(n_axis, n_axis, -(-1024 // (n_axis * n_axis))), cell_count=1024,
                           spacing=float(spacing), smoothing_radius=0.1, emitter_world=W.translation((0, 0.5, 0)))
    pos, vel = oracle.emit(params, 1024)
    pos, vel = oracle.step(params, pos, vel, 1.0 / 60.0, threads=4, frames=120)
    low = pos[pos[:, 1] < 0.2]
    assert len(low) > 0
    mean = float(low[:, 3].astype(np.float64).mean())
    assert params.rest_density * 0.6 < mean < params.rest_density * 1.6


def test_worker_count_does_not_change_bits(oracle):
    # fluid_test.cpp:130-150: 8 workers vs none, 1024 particles, 150 frames.
    params = W.reference_test_scene(1024)
    pos, vel = oracle.emit(params, 1024)
    a = oracle.step(params, pos, vel, 1.0 / 60.0, threads=8, frames=150)
    b = oracle.step(params, pos, vel, 1.0 / 60.0, threads=1, frames=150)
    assert np.array_equal(a[0].view(np.uint32), b[0].view(np.uint32))
    assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


def test_parameter_derivation(oracle):
    # fluid_test.cpp:181-194.
    s = abi.SphFluidSettings()
    for a in range(3):
        s.emitter_half_extents[a] = 0.5
    s.particle_radius, s.rest_density, s.smoothing_radius = 0.05, 1000.0, 0.01
    s.stiffness, s.viscosity = 50.0, 0.5
    params = oracle.derive_params(s, np.array(W.translation((0, 1, 0)), np.float32), 100, 1024)
    assert abs(params.spacing - 0.1) < 1e-6
    assert abs(params.particle_mass - 1000.0 * 0.001) < 1e-4
    assert params.smoothing_radius >= params.spacing
    assert params.cell_count == 1024


def test_substep_bounds(oracle):
    # fluid_test.cpp:196-207.
    params = W.reference_test_scene(100)
    params.smoothing_radius = 0.1
    params.stiffness = 50.0
    assert oracle.fluid_substeps(params, 0.0) == 1
    params.stiffness = 100000.0
    assert oracle.fluid_substeps(params, 1.0 / 60.0) == 8
    params.stiffness = 1.0
    params.smoothing_radius = 10.0
    assert oracle.fluid_substeps(params, 1.0 / 60.0) == 1
    assert oracle.fluid_substeps(params, 100.0) <= 8


def test_grid_against_brute_force_neighbours(oracle):
    """Every in-range pair the brute force finds is reached through the 27
    buckets, with the first 32 ids per bucket (no overflow in this case)."""
    params = W.make_params(container_min=(0, 0, 0), container_max=(0.4, 0.4, 0.4), lattice=(8, 8, 8),
                           cell_count=1024)
    pos, _ = W.jittered_block(params, 512, seed=2)
    cell_of, counts, slots = oracle.grid_build(params, pos)
    assert counts.max() <= 32
    h = np.float32(params.smoothing_radius)
    d = pos[:, None, :3] - pos[None, :, :3]
    r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    brute = (r2 < h * h).sum(axis=1)
    p, q = oracle.pair_counts(params, pos)
    assert q >= brute.sum()  # duplicates of colliding buckets can only add


def test_oracle_instances_match_the_host_construction(oracle):
    """The oracle's instance writer (fluid.cpp:402-466) against the records
    built from the reference's formulas: model = scale(translate(I, p), r),
    identity normal matrix, no joints, and the TLAS row-major transform."""
    from computer_graphics_lab_00_gb300 import abi

    rng = np.random.default_rng(3)
    n = 300
    pos = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
    prev = rng.uniform(-1, 1, (n, 4)).astype(np.float32)
    r = np.float32(0.025)
    inst = np.zeros(n + 4, abi.INSTANCE)
    tlas = np.zeros(n + 1, abi.TLAS_INSTANCE)
    oracle.write_instances(pos, prev, r, inst, 4, 9, tlas, 1, 77, 0, abi.SPH_INSTANCES_WRITE_TLAS, threads=3)
    got = inst[4:]
    for key, src in (("model", pos), ("previous_model", prev)):
        m = np.zeros((n, 16), np.float32)
        m[:, 0] = m[:, 5] = m[:, 10] = r
        m[:, 12:15] = src[:, :3]
        m[:, 15] = 1.0
        assert np.array_equal(got[key], m)
    assert np.array_equal(got["normal_matrix"], np.tile(np.eye(4, dtype=np.float32).reshape(16), (n, 1)))
    assert (got["mesh_index"] == 9).all() and (got["joint_offset"] == 0xFFFFFFFF).all()
    assert (got["skinned_vertex_offset"] == 0xFFFFFFFF).all() and (got["bucket"] == 0).all()
    assert not inst[:4].view(np.uint8).any()
    t = tlas[1:]
    rows = np.zeros((n, 12), np.float32)
    rows[:, 0] = rows[:, 5] = rows[:, 10] = r
    rows[:, 3], rows[:, 7], rows[:, 11] = pos[:, 0], pos[:, 1], pos[:, 2]
    assert np.array_equal(t["transform"], rows)
    assert np.array_equal(t["custom_index_mask"], (np.arange(n) + 4) | (0xFF << 24))
    assert (t["blas"] == 77).all()
    # History reset: the previous model is the current one.
    oracle.write_instances(pos, None, r, inst, 0, 9, flags=abi.SPH_INSTANCES_RESET_HISTORY)
    assert np.array_equal(inst["previous_model"][:n], inst["model"][:n])

