"""CUDA path vs the CPU oracle, through the C ABI (libsph_gb300.so).

Bar: bit-exact. Grid keys, bucket counts and bucket order are integer work;
density, pressure, positions and velocities are compared by their IEEE bit
patterns, because the kernels perform the reference's float operations in
the reference's order (src/physics/fluid_sph.cpp:190-309).
"""
from __future__ import annotations

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import abi
from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

pytestmark = pytest.mark.gpu


def bits(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32).view(np.uint32)


def assert_bit_exact(gpu, ref, what: str) -> None:
    g, r = bits(gpu), bits(ref)
    if not np.array_equal(g, r):
        bad = np.argwhere(g != r)
        i = tuple(bad[0])
        raise AssertionError(
            f"{what}: {len(bad)} words differ; first at {i}: gpu {np.asarray(gpu)[i]!r} oracle {np.asarray(ref)[i]!r}"
        )


def assert_grid_equal(gpu_grid, ref_grid) -> None:
    cell_of, counts, slots = gpu_grid
    o_cell_of, o_counts, o_slots = ref_grid
    np.testing.assert_array_equal(cell_of, o_cell_of)
    np.testing.assert_array_equal(counts, o_counts)
    filled = np.minimum(counts, 32)
    used = (np.arange(32)[None, :] < filled[:, None]).reshape(-1)
    np.testing.assert_array_equal(slots[used], o_slots[used])


def small_block(n: int, lattice, box=(0.6, 0.6, 0.6), cells=None, seed=1):
    params = W.make_params(
        container_min=(0.0, 0.0, 0.0),
        container_max=box,
        lattice=lattice,
        cell_count=cells or W.cell_count_for(n),
    )
    pos, vel = W.jittered_block(params, n, seed)
    return params, pos, vel


@pytest.fixture(scope="module")
def case16k():
    case = W.dam_break_16k()
    pos, vel = case.initial_state()
    return case, pos, vel


def test_grid_bit_exact_16k(native, oracle, case16k):
    case, pos, vel = case16k
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        solver.build_grid()
        assert_grid_equal(solver.grid(), oracle.grid_build(case.params, pos))


def test_one_substep_bit_exact_16k(native, oracle, case16k):
    case, pos, vel = case16k
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        solver.substep(case.dt)
        gp, gv = solver.state()
        # The grid the substep used is the one built from its start positions.
        assert_grid_equal(solver.grid(), oracle.grid_build(case.params, pos))
    op, ov = oracle.substep(case.params, pos, vel, case.dt, threads=oracle.hardware_threads)
    assert_bit_exact(gp[:, 3], op[:, 3], "density")
    assert_bit_exact(gv[:, 3], ov[:, 3], "pressure")
    assert_bit_exact(gp, op, "positions")
    assert_bit_exact(gv, ov, "velocities")


def test_dam_break_16k_600_steps_bit_exact(native, oracle, case16k):
    """The whole 16,384-particle dam break (dt = 1/600, 600 steps) stays
    bit-identical to the oracle, so its density and centre-of-mass
    statistics are identical too."""
    case, pos, vel = case16k
    threads = oracle.hardware_threads
    op, ov = pos, vel
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        for chunk in range(6):
            solver.run(case.dt, 100)
            op, ov = oracle.run_substeps(case.params, op, ov, case.dt, 100, threads=threads)
            gp, gv = solver.state()
            assert_bit_exact(gp, op, f"positions after {(chunk + 1) * 100} steps")
            assert_bit_exact(gv, ov, f"velocities after {(chunk + 1) * 100} steps")
        gs = solver.stats()
    os_ = oracle.stats(case.params, op, ov)
    assert gs.mean_density == pytest.approx(os_.mean_density, rel=1e-12)
    for a in range(3):
        assert gs.centre_of_mass[a] == pytest.approx(os_.centre_of_mass[a], rel=1e-12)
    assert gs.nonfinite == 0


def test_reference_scene_emit_and_frames(native, oracle):
    """tests/fluid_test.cpp:130-150 scene: emit, then frames of 1/60 s (3 substeps each)."""
    params = W.reference_test_scene(1024)
    with FluidSolverGpu(params, 1024) as solver:
        solver.emit(params, 1024)
        gp, gv = solver.state()
        op, ov = oracle.emit(params, 1024)
        assert_bit_exact(gp, op, "emit positions")
        assert_bit_exact(solver.previous_particles()[:, :3], op[:, :3], "previous after emit")
        for _ in range(30):
            solver.step(params, 1.0 / 60.0)
        gp, gv = solver.state()
    op, ov = oracle.step(params, op, ov, 1.0 / 60.0, frames=30)
    assert_bit_exact(gp, op, "positions after 30 frames")
    assert_bit_exact(gv, ov, "velocities after 30 frames")


@pytest.mark.parametrize("n", [1, 2, 31, 33, 127, 4095, 4096, 4097, 10007])
def test_ragged_counts_bit_exact(native, oracle, n):
    lattice = (16, 16, max(1, (n + 255) // 256))
    params, pos, vel = small_block(n, lattice)
    with FluidSolverGpu(params, n) as solver:
        solver.upload(pos, vel)
        solver.run(1.0 / 600.0, 3)
        gp, gv = solver.state()
        assert_grid_equal(solver.grid(), oracle.grid_build(params, oracle.run_substeps(params, pos, vel, 1 / 600.0, 2)[0]))
    op, ov = oracle.run_substeps(params, pos, vel, 1.0 / 600.0, 3)
    assert_bit_exact(gp, op, f"positions n={n}")
    assert_bit_exact(gv, ov, f"velocities n={n}")


@pytest.mark.parametrize("variant,sort", [(4, 1), (6, 1), (4, 2), (4, 0)])
def test_overflowing_bucket_keeps_first_32_ids(native, oracle, variant, sort):
    """More than 32 particles in one cell: only the first 32 by id are
    neighbours (fluid_sph.cpp:179-187); counts stay un-truncated."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(1.0, 1.0, 1.0),
                           lattice=(4, 4, 8), cell_count=1024)
    rng = np.random.default_rng(7)
    n = 300
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (0.481 + rng.uniform(0.0, 0.038, size=(n, 3))).astype(np.float32)  # inside cell [0.48, 0.52)
    pos[200:, :3] = rng.uniform(0.1, 0.9, size=(100, 3)).astype(np.float32)
    pos[:, 3] = 1000.0
    vel = np.zeros((n, 4), np.float32)
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(neighbour_kernel=variant, sort=sort)
        solver.upload(pos, vel)
        solver.build_grid()
        grid = solver.grid()
        ref = oracle.grid_build(params, pos)
        assert_grid_equal(grid, ref)
        assert grid[1].max() >= 200
        solver.substep(1.0 / 600.0)
        gp, gv = solver.state()
    op, ov = oracle.substep(params, pos, vel, 1.0 / 600.0)
    assert_bit_exact(gp, op, "positions with an overflowing bucket")
    assert_bit_exact(gv, ov, "velocities with an overflowing bucket")


@pytest.mark.parametrize("sort", [1, 2])
def test_one_crowded_cell(native, oracle, sort):
    """3,000 of 3,100 particles in one cell: the counting placement ranks a
    bucket past 64 members only until it has found 32 smaller ids, and must
    still put the 32 smallest first in order; the grid and a substep equal
    the oracle's."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(1.0, 1.0, 1.0),
                           lattice=(4, 4, 8), cell_count=1024)
    rng = np.random.default_rng(11)
    n = 3100
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (0.481 + rng.uniform(0.0, 0.038, size=(n, 3))).astype(np.float32)
    pos[rng.permutation(n)[:100], :3] = rng.uniform(0.1, 0.9, size=(100, 3)).astype(np.float32)
    pos[:, 3] = 1000.0
    vel = np.zeros((n, 4), np.float32)
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(sort=sort)
        solver.upload(pos, vel)
        solver.build_grid()
        grid = solver.grid()
        assert grid[1].max() >= 2900
        solver.substep(1.0 / 600.0)
        gp, gv = solver.state()
    assert_grid_equal(grid, oracle.grid_build(params, pos))
    op, ov = oracle.substep(params, pos, vel, 1.0 / 600.0)
    assert_bit_exact(gp, op, "positions with a crowded cell")
    assert_bit_exact(gv, ov, "velocities with a crowded cell")


@pytest.mark.parametrize("crowd", [1, 2, 31, 32, 33, 64, 65, 100])
def test_counting_placement_at_its_size_boundaries(native, oracle, crowd):
    """One cell holding `crowd` particles among scattered others: buckets of
    up to 64 members are ranked in full, larger ones until 32 smaller ids are
    found, and past 32 the rest of the bucket follows in any order; each size
    at those edges gives the oracle's grid (counts and first 32 ids in order)
    and substep."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(1.0, 1.0, 1.0),
                           lattice=(4, 4, 8), cell_count=1024)
    rng = np.random.default_rng(100 + crowd)
    n = 400 + crowd
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.05, 0.95, size=(n, 3)).astype(np.float32)
    crowded = rng.permutation(n)[:crowd]
    pos[crowded, :3] = (0.481 + rng.uniform(0.0, 0.038, size=(crowd, 3))).astype(np.float32)
    pos[:, 3] = 1000.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.normal(0.0, 0.1, size=(n, 3)).astype(np.float32)
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(sort=2)
        solver.upload(pos, vel)
        solver.build_grid()
        grid = solver.grid()
        assert grid[1].max() >= crowd
        solver.substep(1.0 / 600.0)
        gp, gv = solver.state()
    assert_grid_equal(grid, oracle.grid_build(params, pos))
    op, ov = oracle.substep(params, pos, vel, 1.0 / 600.0)
    assert_bit_exact(gp, op, f"positions, {crowd} in one cell")
    assert_bit_exact(gv, ov, f"velocities, {crowd} in one cell")


@pytest.mark.parametrize("schedule", [1, 2])
def test_curve_grid_with_particles_outside_the_box(native, oracle, schedule):
    """Particles uploaded outside the container: the counting placement
    buckets them by their (wrapped) cells' hash and the processing order
    clamps their cells onto the curve's edge; the grid and the substep still
    equal the oracle's."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(1.0, 1.0, 1.0),
                           lattice=(8, 8, 16), cell_count=4096)
    rng = np.random.default_rng(7 + schedule)
    n = 2000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = rng.uniform(0.05, 0.95, size=(n, 3)).astype(np.float32)
    out = rng.permutation(n)[:300]
    pos[out, :3] = rng.uniform(-0.6, 1.6, size=(300, 3)).astype(np.float32)
    pos[:, 3] = 1000.0
    vel = np.zeros((n, 4), np.float32)
    vel[:, :3] = rng.normal(0.0, 0.2, size=(n, 3)).astype(np.float32)
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(sort=2, schedule=schedule)
        solver.upload(pos, vel)
        solver.build_grid()
        grid = solver.grid()
        solver.substep(1.0 / 600.0)
        gp, gv = solver.state()
    assert_grid_equal(grid, oracle.grid_build(params, pos))
    op, ov = oracle.substep(params, pos, vel, 1.0 / 600.0)
    assert_bit_exact(gp, op, "positions with particles outside the box")
    assert_bit_exact(gv, ov, "velocities with particles outside the box")


@pytest.mark.parametrize("variant,schedule", [(4, 1), (6, 1), (6, 0)])
def test_hash_collisions_and_duplicate_buckets(native, oracle, variant, schedule):
    """With few buckets, neighbour cells collide and the same bucket is
    visited twice for one particle; the reference counts it twice and so
    must the kernels (the staged integrate copies such a bucket once and
    reads it for both neighbours)."""
    n = 8192
    params, pos, vel = small_block(n, (16, 16, 32), box=(0.5, 0.8, 0.8), cells=1024)
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(neighbour_kernel=variant, schedule=schedule)
        solver.upload(pos, vel)
        solver.run(1.0 / 600.0, 5)
        gp, gv = solver.state()
    op, ov = oracle.run_substeps(params, pos, vel, 1.0 / 600.0, 5, threads=oracle.hardware_threads)
    assert_bit_exact(gp, op, "positions with collisions")
    assert_bit_exact(gv, ov, "velocities with collisions")


def test_pair_counts_match_oracle(native, oracle, case16k):
    case, pos, vel = case16k
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        st = solver.stats()
    p, q = oracle.pair_counts(case.params, pos)
    assert st.candidates == p
    assert st.pairs_in_range == q


def test_1m_grid_and_two_substeps_bit_exact(native, oracle):
    """The 1,048,576-particle dam break (C = 2^21): grid and two substeps."""
    case = W.dam_break_1m()
    pos, vel = case.initial_state()
    threads = oracle.hardware_threads
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        solver.build_grid()
        assert_grid_equal(solver.grid(), oracle.grid_build(case.params, pos, threads=threads))
        solver.run(case.dt, 2)
        gp, gv = solver.state()
    op, ov = oracle.run_substeps(case.params, pos, vel, case.dt, 2, threads=threads)
    assert_bit_exact(gp, op, "1M positions")
    assert_bit_exact(gv, ov, "1M velocities")


def test_1m_compressed_state_bit_exact(native, oracle):
    """The 1M dam break 300 substeps in (collapsing and compressed, so many
    particles pass integrate's 32-entry lists and drain mid-walk, and the
    Morton order is several substeps stale): two more substeps from the GPU's
    own state equal the oracle's from the same state, and the pair counts
    agree."""
    case = W.dam_break_1m()
    pos, vel = case.initial_state()
    threads = oracle.hardware_threads
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.upload(pos, vel)
        solver.run(case.dt, 300)
        sp, sv = solver.state()
        st = solver.stats()
        assert st.pairs_in_range > 30 * case.count  # denser than the lattice (29.3 per particle)
        p, q = oracle.pair_counts(case.params, sp, threads=threads)
        assert (st.candidates, st.pairs_in_range) == (p, q)
        solver.run(case.dt, 2)
        gp, gv = solver.state()
    op, ov = oracle.run_substeps(case.params, sp, sv, case.dt, 2, threads=threads)
    assert_bit_exact(gp, op, "1M positions from the compressed state")
    assert_bit_exact(gv, ov, "1M velocities from the compressed state")


@pytest.mark.parametrize("mass", [0.0, -0.3])
def test_nonpositive_mass_matches_oracle(native, oracle, mass):
    """Density drops out-of-range terms with a NaN-keeping max while mass and
    the poly6 constant are positive, and with the reference's select
    otherwise; a zero or negative particle mass takes the second form."""
    n = 4096
    params, pos, vel = small_block(n, (16, 16, 16), box=(0.5, 0.5, 0.5), cells=W.cell_count_for(n))
    params.gravity[3] = mass
    with FluidSolverGpu(params, n) as solver:
        solver.upload(pos, vel)
        solver.run(1.0 / 600.0, 2)
        gp, gv = solver.state()
    op, ov = oracle.run_substeps(params, pos, vel, 1.0 / 600.0, 2)
    assert_bit_exact(gp, op, f"positions, mass {mass}")
    assert_bit_exact(gv, ov, f"velocities, mass {mass}")


def test_gpu_runs_are_deterministic(native):
    case = W.dam_break_16k()
    pos, vel = case.initial_state()
    out = []
    for _ in range(2):
        with FluidSolverGpu(case.params, case.count) as solver:
            solver.upload(pos, vel)
            solver.run(case.dt, 50)
            out.append(solver.state())
    assert_bit_exact(out[0][0], out[1][0], "run-to-run positions")
    assert_bit_exact(out[0][1], out[1][1], "run-to-run velocities")


def test_errors_are_status_codes(native):
    case = W.dam_break_16k()
    bad = case.params.copy()
    bad.lattice[3] = 1000  # not a power of two
    with pytest.raises(abi.SphError) as e:
        FluidSolverGpu(bad, 16)
    assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT
    with FluidSolverGpu(case.params, 16) as solver:
        pos = np.zeros((17, 4), np.float32)
        with pytest.raises(abi.SphError) as e:
            solver.upload(pos)
        assert e.value.status == abi.SPH_ERR_CAPACITY
        pos = np.zeros((4, 4), np.float32)
        pos[2, 1] = np.nan
        with pytest.raises(abi.SphError) as e:
            solver.upload(pos)
        assert e.value.status == abi.SPH_ERR_NONFINITE
        solver.upload(np.zeros((0, 4), np.float32))
        solver.step(case.params, 1.0 / 60.0)  # empty: no-op, like FluidSolver::step
        assert solver.particles().shape == (0, 4)
        with pytest.raises(abi.SphError) as e:
            solver.substep(-1.0)
        assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT
    bad = case.params.copy()
    bad.collider_count = 9
    with pytest.raises(abi.SphError) as e:
        FluidSolverGpu(bad, 16)
    assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT
    bad = case.params.copy()
    bad.collider_count = 1
    bad.colliders[0].type = 6
    with pytest.raises(abi.SphError) as e:
        FluidSolverGpu(bad, 16)
    assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT
    bad = case.params.copy()
    bad.field_count = 9
    with pytest.raises(abi.SphError) as e:
        FluidSolverGpu(bad, 16)
    assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("tuning", [
    dict(neighbour_kernel=0, block_size=128, queue_depth=16, radix_bits=7, schedule=0, sort=0),
    dict(neighbour_kernel=0, block_size=128, queue_depth=16, radix_bits=7, schedule=1, sort=0),
    dict(neighbour_kernel=1, block_size=64, queue_depth=8, radix_bits=8, schedule=1, sort=0),
    dict(neighbour_kernel=1, block_size=128, queue_depth=16, radix_bits=7, schedule=0, sort=0),
    dict(neighbour_kernel=1, block_size=256, queue_depth=24, radix_bits=5, schedule=1, sort=0),
    dict(neighbour_kernel=1, block_size=128, queue_depth=32, radix_bits=3, schedule=0, sort=0),
    dict(neighbour_kernel=2, block_size=64, queue_depth=16, radix_bits=7, schedule=1, sort=0),
    dict(neighbour_kernel=2, block_size=128, queue_depth=16, radix_bits=8, schedule=0, sort=0),
    dict(neighbour_kernel=3, block_size=128, queue_depth=16, radix_bits=7, schedule=1, sort=0),
    dict(neighbour_kernel=3, block_size=256, queue_depth=16, radix_bits=6, schedule=0, sort=0),
    dict(neighbour_kernel=4, block_size=64, queue_depth=16, radix_bits=7, schedule=0, sort=0),
    dict(neighbour_kernel=4, block_size=128, queue_depth=16, radix_bits=7, schedule=1, sort=0),
    dict(neighbour_kernel=4, block_size=256, queue_depth=16, radix_bits=8, schedule=1, sort=0),
    dict(neighbour_kernel=4, block_size=256, queue_depth=32, radix_bits=6, schedule=0, sort=1),
    dict(neighbour_kernel=3, block_size=128, queue_depth=16, radix_bits=6, schedule=1, sort=1),
    dict(neighbour_kernel=0, block_size=128, queue_depth=16, radix_bits=6, schedule=0, sort=1),
    dict(neighbour_kernel=5, block_size=128, queue_depth=16, radix_bits=7, schedule=0, sort=0),
    dict(neighbour_kernel=5, block_size=128, queue_depth=16, radix_bits=8, schedule=1, sort=0),
    dict(neighbour_kernel=5, block_size=128, queue_depth=32, radix_bits=6, schedule=1, sort=1),
    dict(neighbour_kernel=5, block_size=256, queue_depth=32, radix_bits=6, schedule=0, sort=1),
    dict(neighbour_kernel=4, block_size=128, queue_depth=16, radix_bits=7, schedule=2, sort=1),
    dict(neighbour_kernel=3, block_size=256, queue_depth=16, radix_bits=6, schedule=2, sort=0),
    dict(neighbour_kernel=5, block_size=128, queue_depth=16, radix_bits=8, schedule=2, sort=1),
    dict(neighbour_kernel=6, block_size=128, queue_depth=16, radix_bits=8, schedule=1, sort=1),
    dict(neighbour_kernel=6, block_size=256, queue_depth=16, radix_bits=7, schedule=2, sort=1),
    dict(neighbour_kernel=6, block_size=128, queue_depth=16, radix_bits=6, schedule=0, sort=0),
    dict(neighbour_kernel=6, block_size=256, queue_depth=32, radix_bits=8, schedule=1, sort=0),
    dict(neighbour_kernel=4, block_size=128, queue_depth=16, radix_bits=7, schedule=1, sort=2),
    dict(neighbour_kernel=4, block_size=128, queue_depth=16, radix_bits=7, schedule=0, sort=2),
    dict(neighbour_kernel=6, block_size=128, queue_depth=16, radix_bits=7, schedule=2, sort=2),
    dict(neighbour_kernel=1, block_size=128, queue_depth=16, radix_bits=7, schedule=1, sort=2),
])
def test_launch_shapes_do_not_change_bits(native, oracle, tuning):
    """Every launch shape the autotuner may pick gives the oracle's bits."""
    n = 8192
    params, pos, vel = small_block(n, (16, 16, 32), box=(0.5, 0.8, 0.8), cells=W.cell_count_for(n))
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(**tuning)
        assert solver.tuning() == tuning
        solver.upload(pos, vel)
        solver.run(1.0 / 600.0, 4)
        gp, gv = solver.state()
    op, ov = oracle.run_substeps(params, pos, vel, 1.0 / 600.0, 4, threads=oracle.hardware_threads)
    assert_bit_exact(gp, op, f"positions {tuning}")
    assert_bit_exact(gv, ov, f"velocities {tuning}")


def test_morton_order_across_remakes_and_count_changes(native, oracle):
    """The Morton processing order is remade every 8 grid builds and after a
    change of particle count, and kept across an upload of the same count (a
    stale order); the bits stay the oracle's throughout, through graph runs
    and the direct grid build."""
    n = 8192
    dt = 1.0 / 600.0
    params, pos, vel = small_block(n, (16, 16, 32), box=(0.5, 0.8, 0.8), cells=W.cell_count_for(n))
    threads = oracle.hardware_threads
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(schedule=1)
        solver.upload(pos, vel)
        solver.run(dt, 15)
        solver.build_grid()
        solver.run(dt, 22)
        gp, gv = solver.state()
        op, ov = oracle.run_substeps(params, pos, vel, dt, 37, threads=threads)
        assert_bit_exact(gp, op, "positions after 37 substeps")
        assert_bit_exact(gv, ov, "velocities after 37 substeps")
        # Same count, unrelated positions: the order is stale, not wrong.
        solver.upload(pos[::-1].copy(), vel[::-1].copy())
        solver.run(dt, 3)
        gp, gv = solver.state()
        op, ov = oracle.run_substeps(params, pos[::-1].copy(), vel[::-1].copy(), dt, 3, threads=threads)
        assert_bit_exact(gp, op, "positions after a same-count upload")
        assert_bit_exact(gv, ov, "velocities after a same-count upload")
        op, ov = oracle.run_substeps(params, pos, vel, dt, 37, threads=threads)
        m = 5000
        solver.upload(op[:m], ov[:m])
        solver.run(dt, 18)
        gp, gv = solver.state()
        op, ov = oracle.run_substeps(params, op[:m], ov[:m], dt, 18, threads=threads)
        assert_bit_exact(gp, op, "positions after the count change")
        assert_bit_exact(gv, ov, "velocities after the count change")


@pytest.mark.parametrize("sort,bits", [(1, 6), (0, 5), (0, 8), (2, 6)])
def test_grid_sorts_agree_at_one_million(native, oracle, sort, bits):
    """The one-sweep sort (3 look-back passes over 21-bit keys at 1M) and the
    three-kernel passes give the oracle's grid bit for bit."""
    case = W.dam_break_1m()
    pos, vel = case.initial_state()
    with FluidSolverGpu(case.params, case.count) as solver:
        solver.set_tuning(sort=sort, radix_bits=bits)
        solver.upload(pos, vel)
        solver.build_grid()
        got = solver.grid()
    assert_grid_equal(got, oracle.grid_build(case.params, pos, threads=oracle.hardware_threads))


def test_grid_and_substeps_past_256_sort_tiles(native, oracle):
    """2,064,384 particles (504 sort tiles): the one-sweep passes add whole
    32-tile chunk sums before their own chunk's tiles. The grid and two
    substeps (Morton order, whose keys take the same sort) are the oracle's."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(4.0, 3.0, 2.0), lattice=(192, 128, 84),
                           cell_count=W.cell_count_uncapped(192 * 128 * 84))
    n = 192 * 128 * 84
    pos, vel = W.jittered_block(params, n, seed=4)
    threads = oracle.hardware_threads
    with FluidSolverGpu(params, n) as solver:
        solver.set_tuning(sort=1)
        solver.upload(pos, vel)
        solver.build_grid()
        got = solver.grid()
        solver.run(1.0 / 600.0, 2)
        gp, gv = solver.state()
    assert_grid_equal(got, oracle.grid_build(params, pos, threads=threads))
    op, ov = oracle.run_substeps(params, pos, vel, 1.0 / 600.0, 2, threads=threads)
    assert_bit_exact(gp, op, "positions past 256 sort tiles")
    assert_bit_exact(gv, ov, "velocities past 256 sort tiles")


def test_bad_tuning_is_rejected(native):
    case = W.dam_break_16k()
    with FluidSolverGpu(case.params, 16) as solver:
        for bad in (dict(block_size=100), dict(queue_depth=12), dict(neighbour_kernel=7), dict(neighbour_kernel=6, block_size=64),
                    dict(radix_bits=0),
                    dict(radix_bits=9), dict(schedule=3), dict(sort=3)):
            with pytest.raises(abi.SphError) as e:
                solver.set_tuning(**bad)
            assert e.value.status == abi.SPH_ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("mode,count", [(0, 1 << 29), (1, 1 << 30), (2, 1 << 26), (3, 1 << 26), (4, 1 << 26),
                                        pytest.param(5, 1 << 26, marks=pytest.mark.xfail(
                                            reason="ptxas contracts packed f32x2 mul+add into a fused "
                                                   "multiply-add even under --fmad=false, so the exact passes "
                                                   "use scalar arithmetic", strict=False))])
def test_reciprocal_division_matches_ieee(native, mode, count):
    """Arithmetic the exact passes rely on, against IEEE scalar operations:
    division through a correctly rounded reciprocal (modes 0-1: every divisor
    mantissa; random operands over 2^-60..2^60), and packed f32x2 mul, add and
    sub lane by lane (modes 2-4). Mode 5 records that a packed squared-distance
    chain does not round like the scalar chain."""
    import ctypes

    case = W.dam_break_16k()
    with FluidSolverGpu(case.params, 16) as solver:
        bad = ctypes.c_uint64()
        status = native.sph_selftest_division(solver._ctx, 12345, count, mode, ctypes.byref(bad))
        assert status == 0
        assert bad.value == 0


def _sweep_mismatches(native, x_from, x_to, y):
    """Dividends x in [x_from, x_to) (every float), divisor y: how many
    quotients through the reciprocal differ from IEEE division."""
    import ctypes

    lo = int(np.array([x_from], np.float32).view(np.uint32)[0])
    hi = int(np.array([x_to], np.float32).view(np.uint32)[0])
    yb = int(np.array([y], np.float32).view(np.uint32)[0])
    bad = ctypes.c_uint64()
    with FluidSolverGpu(W.dam_break_16k().params, 16) as solver:
        assert native.sph_selftest_division(solver._ctx, (lo << 32) | yb, hi - lo, 6, ctypes.byref(bad)) == 0
    return bad.value


@pytest.mark.parametrize("divisor", [0.04 * 0.04, 0.1 * 0.1, 1.0, 998.3, 3.7e-5])
def test_reciprocal_division_floor(native, divisor):
    """Exhaustive over one divisor: division through the correctly rounded
    reciprocal equals IEEE division for every dividend from 2^-100 up to the
    divisor, the floor the exact passes rely on (their dividends stay far
    above it)."""
    y = np.float32(divisor)
    assert _sweep_mismatches(native, np.float32(2.0 ** -100), y, y) == 0


def test_reciprocal_division_below_the_floor_can_differ(native):
    """Below about 2^-105 the FMA residual underflows and some quotients are
    one ulp off IEEE division: the reason for the floor."""
    y = np.float32(0.04) * np.float32(0.04)
    assert _sweep_mismatches(native, np.float32(0.0), np.float32(2.0 ** -100), y) > 0


def test_pair_list_overflow_falls_back_bit_exact(native, oracle):
    """Particles with more in-range pairs than a list holds (64) are scanned
    directly by integrate; a compressed clump forces that path."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(1.0, 1.0, 1.0),
                           lattice=(4, 4, 8), cell_count=4096)
    rng = np.random.default_rng(3)
    n = 2000
    pos = np.zeros((n, 4), np.float32)
    pos[:, :3] = (0.4 + rng.uniform(0.0, 0.12, size=(n, 3))).astype(np.float32)
    pos[:, 3] = 1000.0
    vel = np.zeros((n, 4), np.float32)
    for variant, schedule, block, queue in ((2, 0, 256, 32), (3, 1, 256, 32), (4, 0, 256, 32), (4, 1, 256, 32),
                                            (4, 0, 256, 24), (4, 0, 256, 16), (4, 0, 128, 32), (4, 0, 64, 32),
                                            (5, 0, 128, 32), (5, 1, 128, 32), (6, 0, 128, 32), (6, 1, 128, 32),
                                            (6, 2, 256, 32)):
        with FluidSolverGpu(params, n) as solver:
            solver.set_tuning(neighbour_kernel=variant, schedule=schedule, block_size=block, queue_depth=queue)
            solver.upload(pos, vel)
            solver.run(1.0 / 600.0, 2)
            gp, gv = solver.state()
        op, ov = oracle.run_substeps(params, pos, vel, 1.0 / 600.0, 2)
        assert_bit_exact(gp, op, f"positions with list overflow, variant {variant}")
        assert_bit_exact(gv, ov, f"velocities with list overflow, variant {variant}")


def test_kernel_counter_counts_the_graph_and_the_order_remakes(native):
    """sph_kernels_launched advances by the substep graph's kernels for every
    substep run, plus the processing-order remakes: one tank's order is made
    by counting (five kernels) every third build; the plain bucket order
    (schedule 0) has none."""
    case = W.dam_break_16k()
    with FluidSolverGpu(case.params, case.count) as s:
        s.upload(*case.initial_state())
        s.run(case.dt, 1)
        per = s.launches_per_substep()
        assert per >= 8  # counting grid (5), gather, density, integrate
        before = s.kernels_launched()
        s.run(case.dt, 9)
        assert s.kernels_launched() - before == 9 * per + 3 * 5
        s.set_tuning(schedule=0)
        s.run(case.dt, 1)
        before = s.kernels_launched()
        s.run(case.dt, 6)
        assert s.kernels_launched() - before == 6 * s.launches_per_substep()
