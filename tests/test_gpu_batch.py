"""Batched tanks through the C ABI: every tank must give exactly the bits
the oracle gives for that tank alone (the batch shares launches, not
physics)."""
from __future__ import annotations

import numpy as np
import pytest

from computer_graphics_lab_00_gb300 import workloads as W
from computer_graphics_lab_00_gb300.batch import BatchSolverGpu

pytestmark = pytest.mark.gpu


def same(a, b) -> bool:
    return np.array_equal(np.asarray(a, np.float32).view(np.uint32), np.asarray(b, np.float32).view(np.uint32))


def small_set(tanks=6, seed=4):
    """A few tanks of the batched generator's shape, with small counts."""
    full = W.batched_tanks(tanks=tanks, seed=seed)
    params, counts = [], []
    for t in range(tanks):
        n = 400 + 611 * t
        extent = [full.params[t].container_max[a] for a in range(3)]
        lattice = W.tank_lattice(n, extent, 0.4, 0.02)
        params.append(W.make_params(container_min=(0, 0, 0), container_max=extent, lattice=lattice,
                                    cell_count=W.cell_count_for(n)))
        counts.append(n)
    return W.TankSet("small", params, counts, 1.0 / 600.0, 10, seed)


@pytest.fixture(scope="module")
def tanks():
    return small_set()


def load(ts):
    solver = BatchSolverGpu(ts.params, ts.counts)
    for t in range(len(ts.counts)):
        solver.upload(t, *ts.initial_state(t))
    return solver


@pytest.mark.parametrize("schedule,substeps,sort", [(0, 5, 1), (1, 5, 1), (1, 20, 1), (2, 20, 1), (1, 5, 2), (0, 20, 2)])
def test_each_tank_matches_the_oracle(native, oracle, tanks, schedule, substeps, sort):
    """Sorted and Morton processing orders; 20 substeps cross remakes of the
    Morton order (every 8 grid builds: these tanks' boxes have more cells
    than buckets, so the order sorts curve keys with the tank above the cell
    code)."""
    with load(tanks) as solver:
        solver.set_tuning(schedule=schedule, sort=sort)
        solver.run(tanks.dt, substeps)
        for t in range(len(tanks.counts)):
            gp, gv = solver.download(t)
            op, ov = oracle.run_substeps(tanks.params[t], *tanks.initial_state(t), tanks.dt, substeps)
            assert same(gp, op) and same(gv, ov), f"tank {t}"


@pytest.mark.parametrize("schedule,block", [(1, 128), (2, 256)])
def test_staged_integrate_per_tank(native, oracle, tanks, schedule, block):
    """The shared-memory-staged integrate (blocks that span two tanks, and a
    frozen tank whose particles sit the substep out) matches the oracle in
    every tank."""
    n = len(tanks.counts)
    dt = [1.0 / 600.0] * n
    substeps = [2] * n
    with load(tanks) as solver:
        solver.set_tuning(neighbour_kernel=6, block_size=block, schedule=schedule)
        active = [1] * n
        active[2] = 0
        solver.set_active(active)
        solver.run_per_tank(dt, substeps)
        for t in range(n):
            gp, gv = solver.download(t)
            runs = 0 if t == 2 else substeps[t]
            op, ov = oracle.run_substeps(tanks.params[t], *tanks.initial_state(t), dt[t], runs)
            assert same(gp, op) and same(gv, ov), f"tank {t}"


def test_per_tank_step_lengths_and_frozen_tanks(native, oracle, tanks):
    n = len(tanks.counts)
    dt = [1.0 / 600.0 if t % 2 == 0 else 1.0 / 1200.0 for t in range(n)]
    substeps = [t % 3 for t in range(n)]  # 0, 1, 2, 0, 1, 2
    with load(tanks) as solver:
        active = [1] * n
        active[1] = 0
        solver.set_active(active)
        solver.run_per_tank(dt, substeps)
        for t in range(n):
            gp, gv = solver.download(t)
            runs = 0 if t == 1 else substeps[t]
            op, ov = oracle.run_substeps(tanks.params[t], *tanks.initial_state(t), dt[t], runs)
            assert same(gp, op) and same(gv, ov), f"tank {t}"


def test_few_active_tanks_build_a_compacted_grid(native, oracle, tanks):
    """With at most half the particles active, run() builds the grid over the
    active tanks alone (a compacted id list). The active tanks match the
    oracle, idle tanks keep their bits, and a full run afterwards (every tank
    active again) continues bit-exactly."""
    n = len(tanks.counts)
    states = [tanks.initial_state(t) for t in range(n)]
    with load(tanks) as solver:
        active = [0] * n
        active[0] = 1
        active[3] = 1
        assert tanks.counts[0] + tanks.counts[3] <= sum(tanks.counts) // 2
        solver.set_active(active)
        solver.run(tanks.dt, 4)
        solver.set_active([1] * n)
        solver.run(tanks.dt, 2)
        for t in range(n):
            gp, gv = solver.download(t)
            runs = 6 if active[t] else 2
            op, ov = oracle.run_substeps(tanks.params[t], *states[t], tanks.dt, runs)
            assert same(gp, op) and same(gv, ov), f"tank {t}"


def test_restore_selected_tanks_from_a_snapshot(native, tanks):
    """restore_tanks copies back exactly the selected tanks (adjacent ones in
    one copy) and leaves the others as they ran."""
    n = len(tanks.counts)
    with load(tanks) as solver:
        solver.run(tanks.dt, 2)
        saved = [solver.download(t) for t in range(n)]
        solver.snapshot(1, save=True)
        solver.run(tanks.dt, 3)
        moved = [solver.download(t) for t in range(n)]
        which = [1, 1, 0, 1, 0, 1][:n]
        solver.restore_tanks(1, which)
        for t in range(n):
            gp, gv = solver.download(t)
            want = saved[t] if which[t] else moved[t]
            assert same(gp, want[0]) and same(gv, want[1]), f"tank {t}"
            assert which[t] or not same(gp, saved[t][0])


def test_batch_step_matches_fluid_solver_step(native, oracle, tanks):
    with load(tanks) as solver:
        for _ in range(3):
            solver.step(1.0 / 60.0)
        for t in range(len(tanks.counts)):
            gp, gv = solver.download(t)
            op, ov = oracle.step(tanks.params[t], *tanks.initial_state(t), 1.0 / 60.0, frames=3)
            assert same(gp, op) and same(gv, ov), f"tank {t}"


def test_per_tank_statistics(native, oracle, tanks):
    with load(tanks) as solver:
        solver.run(tanks.dt, 3)
        stats = solver.stats()
        for t in range(len(tanks.counts)):
            op, ov = oracle.run_substeps(tanks.params[t], *tanks.initial_state(t), tanks.dt, 3)
            ref = oracle.stats(tanks.params[t], op, ov)
            assert stats[t].particles == tanks.counts[t]
            assert stats[t].mean_density == pytest.approx(ref.mean_density, rel=1e-12)
            assert stats[t].mean_compression == pytest.approx(ref.mean_compression, rel=1e-9, abs=1e-15)
            for a in range(3):
                assert stats[t].centre_of_mass[a] == pytest.approx(ref.centre_of_mass[a], rel=1e-12)


def test_autotune_restores_state_and_keeps_bits(native, oracle, tanks, tmp_path):
    with load(tanks) as solver:
        before = [solver.download(t) for t in range(len(tanks.counts))]
        result = solver.autotune(tanks.dt, 2, cache=tmp_path / "tune.json", key="small")
        assert result["ms_per_substep"] > 0
        for t, (p, v) in enumerate(before):
            gp, gv = solver.download(t)
            assert same(gp, p) and same(gv, v), f"autotune changed tank {t}"
        solver.run(tanks.dt, 2)
        for t in range(len(tanks.counts)):
            gp, gv = solver.download(t)
            op, ov = oracle.run_substeps(tanks.params[t], *tanks.initial_state(t), tanks.dt, 2)
            assert same(gp, op) and same(gv, ov), f"tank {t} after autotune"
        cached = solver.autotune(tanks.dt, 2, cache=tmp_path / "tune.json", key="small")
        assert cached["tuning"] == result["tuning"]


def test_256_tank_workload_spot_checks(native, oracle):
    """The full 256-tank set (about 5M particles): two substeps, four tanks
    checked against the oracle."""
    ts = W.batched_tanks()
    with BatchSolverGpu(ts.params, ts.counts) as solver:
        for t in range(len(ts.counts)):
            solver.upload(t, *ts.initial_state(t))
        solver.run(ts.dt, 2)
        for t in (0, 17, 128, 255):
            gp, gv = solver.download(t)
            op, ov = oracle.run_substeps(ts.params[t], *ts.initial_state(t), ts.dt, 2,
                                         threads=oracle.hardware_threads)
            assert same(gp, op) and same(gv, ov), f"tank {t}"


def cell_bins(ts) -> tuple[int, int]:
    """The batch processing order's cell bins (each tank's cells a side from
    its low corner) against the batch's buckets."""
    bins = 0
    for p in ts.params:
        h = np.float32(p.smoothing_radius)
        r = np.float32(p.particle_radius)
        cells = 1
        for a in range(3):
            lo = np.floor(np.float32(p.container_min[a] + r) / h)
            hi = np.floor(np.float32(p.container_max[a] - r) / h)
            cells *= int(max(hi - lo + 1, 1))
        bins += cells
    return bins, sum(int(p.cell_count) for p in ts.params)


@pytest.mark.parametrize("wide", [False, True])
def test_batch_processing_order_by_cells_or_by_sorted_keys(native, oracle, wide):
    """A batch's curve order: each tank's cells in row order by counting when
    the cells fit the buckets, else sorted curve keys (wide tanks: boxes far
    larger than their fluid). Either way, across order remakes, every tank
    equals the oracle's run of it alone."""
    counts = [900, 1700, 2600, 4100]
    params = []
    for n in counts:
        side = 1.3 * 0.02 * n ** (1.0 / 3.0)  # a box a little larger than the fluid
        box = (3.0, 2.0, 3.0) if wide else (side, side, side)
        lattice = W.tank_lattice(n, (side, side, side), 0.8, 0.02)
        params.append(W.make_params(container_min=(0, 0, 0), container_max=box, lattice=lattice,
                                    cell_count=W.cell_count_for(n)))
    ts = W.TankSet("wide" if wide else "snug", params, counts, 1.0 / 600.0, 10, 9)
    bins, buckets = cell_bins(ts)
    assert (bins > buckets) == wide
    substeps = 10
    with load(ts) as solver:
        solver.set_tuning(schedule=1, sort=2)
        solver.run(ts.dt, substeps)
        for t in range(len(ts.counts)):
            gp, gv = solver.download(t)
            op, ov = oracle.run_substeps(ts.params[t], *ts.initial_state(t), ts.dt, substeps)
            assert same(gp, op) and same(gv, ov), f"tank {t}"
