#!/usr/bin/env python
"""Throughput of the GB300 SPH fluid step on the 1,048,576-particle dam break.

One "step" is one substep of the plain SPH solver (grid build, density and
pressure, forces + integration + walls) over all particles of the tank at
dt = 1/600 s. Inputs are seeded synthetic (jittered emit lattice).

Our arm (default) prints one JSON line with
  value    sim-s x particles / s with the state resident in HBM, device time
           from CUDA events on the solver's stream, L2 flushed before every
           timed substep (a 256 MB write);
  e2e      the same metric through the C ABI with host buffers: every step
           is one sph_step_host call, which uploads the state from pinned
           host memory, runs the substep and downloads the new state;
  roofline the dominant kernel's algorithmic bytes per launch over its
           event-timed duration, against the measured HBM copy bandwidth;
  cpu_baseline  the CPU oracle (a restatement of the reference's CPU solver)
           timed on this host's cores on a bounded sample.
On one GPU it adds the other legs: the whole 1,000-substep run (sustained),
256 batched tanks, the learned 5x-dt step, the tank with shape colliders and
force fields (obstacles), the instance writer and the fluid surface.
`--impl reference` times the reference's CPU solver path (the oracle port,
all host threads) on the same workload and metric.

With torchrun (N > 1) every rank advances its own replica of the tank (the
single-tank step does not shard); value sums particles over ranks and takes
the slowest rank's time.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "sim-s×particles/s @1M: plain vs learned 5×dt (≤1% density err); % HBM peak"
UNIT = "sim-s*particles/s"
FALLBACK_HBM_GBS = 6800.0
FLUSH_BYTES = 256 << 20
WEIGHTS = ROOT / "computer_graphics_lab_00_gb300" / "weights" / "sph_correction.npz"


def parse_args():
    p = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--e2e-steps", type=int, default=None, help="steps of the end-to-end leg (default: --steps)")
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample length")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--surface", action=argparse.BooleanOptionalAction, default=True,
                   help="time the fluid surface (field + marching cubes) beside the step")
    p.add_argument("--batched-steps", type=int, default=20,
                   help="substeps of the 256-tank leg (0 skips it)")
    p.add_argument("--learned-steps", type=int, default=20,
                   help="coarse steps of the learned 5x-dt leg at 1M (0 skips it)")
    p.add_argument("--neighbour-kernel", type=int, default=None,
                   help="neighbour kernel of the 1M tank's legs (sph_tuning.neighbour_kernel; default: the library's)")
    p.add_argument("--learned-eval", action=argparse.BooleanOptionalAction, default=True,
                   help="config 4: 64 held-out tanks of 32,768 over 2 s, learned and plain coarse vs plain fine")
    p.add_argument("--fallback-steps", type=int, default=600,
                   help="config 5: coarse steps of the 1,024 x 8,192 learned-with-fallback leg (0: skip)")
    p.add_argument("--sustained-steps", type=int, default=1000,
                   help="substeps of the whole-run leg of the 1M dam break (0 skips it)")
    p.add_argument("--instance-reps", type=int, default=20,
                   help="timed calls of the instance writer at 1M (0 skips it)")
    p.add_argument("--obstacle-steps", type=int, default=50,
                   help="substeps of the 1M colliders-and-fields leg, and of the plain tank beside it (0 skips it)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def workload_config(case, world: int) -> dict:
    p = case.params
    return {
        "workload": case.name,
        "particles": case.count,
        "dt": case.dt,
        "lattice": [int(p.lattice[0]), int(p.lattice[1]), int(p.lattice[2])],
        "box": [[float(p.container_min[a]) for a in range(3)], [float(p.container_max[a]) for a in range(3)]],
        "buckets": int(p.lattice[3]),
        "smoothing_radius": float(p.smoothing_radius),
        "spacing": float(p.emitter_half_extents[3]),
        "jitter": "uniform +-1e-4 m, splitmix64 seed 0",
        "l2": "flushed before every timed substep (256 MB write); working set ~120 MB",
        "timed_substeps": "spread evenly over the 1,000-substep run (untimed substeps between them)",
        "parallelism": "single tank" if world == 1 else f"{world} replicas (no data exchange)",
    }


def measured_hbm_peak():
    path = ROOT / "MEASURED_PEAKS.json"
    try:
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.file = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        self.file.flush()

    def summary(self) -> dict:
        self.file.seek(0)
        rows = list(csv.reader(io.StringIO(self.file.read())))
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in rows:
            if len(row) < 9:
                continue
            try:
                sm.append(float(row[1]))
                mx.append(float(row[2]))
            except ValueError:
                continue
            for name, flag in zip(names, row[5:9]):
                if flag.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(case, seconds: float) -> dict:
    """The CPU oracle on a bounded sample: whole-tank substeps until `seconds` pass."""
    from oracle.bind import Oracle

    oracle = Oracle()
    threads = oracle.hardware_threads
    pos, vel = case.initial_state()
    start = time.perf_counter()
    steps = 0
    while True:
        pos, vel = oracle.substep(case.params, pos, vel, case.dt, threads=threads)
        steps += 1
        if time.perf_counter() - start >= seconds:
            break
    wall = time.perf_counter() - start
    return {
        "value": case.count * case.dt * steps / wall,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"{steps} substeps of the full {case.count}-particle tank from its initial state ({wall:.1f} s)",
        "ms_per_step": 1e3 * wall / steps,
    }


def batched_leg(steps: int, flush, device: int, world: int = 1) -> dict:
    """256 independent tanks (about 5M particles, uneven sizes) advanced by one
    CUDA graph launch per substep; launch shape from the autotuner. With N
    ranks the tanks are sharded by particle count (no exchange between
    ranks); the time is the slowest rank's and the work is fixed ("strong")."""
    import torch

    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.sharding import ShardedBatch

    ts = W.batched_tanks()
    rank = int(os.environ.get("RANK", "0"))
    shard = ShardedBatch(ts, rank, world, device=device)
    solver = shard.solver
    ms = 0.0
    tune = {"tuning": None}
    phases = {}
    launches = 0
    if solver is not None:
        tune = solver.autotune(ts.dt, 3)
        stream = torch.cuda.ExternalStream(solver.stream(), device=torch.device("cuda", device))
        solver.run(ts.dt, 3)
        solver.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                starts[k].record(stream)
            solver.run(ts.dt, 1)
            ends[k].record(stream)
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / steps
        phases = solver.profile(ts.dt, 3)
        launches = solver.launches_per_substep()
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([ms], dtype=torch.float64, device=f"cuda:{device}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    n = ts.total_particles
    out = {
        "workload": ts.name, "tanks": len(ts.counts), "particles": n, "dt": ts.dt, "steps": steps,
        "ms_per_step": ms, "value": n * ts.dt / (ms / 1e3), "unit": UNIT,
        "particle_steps_per_s": n / (ms / 1e3), "tuning": tune["tuning"],
        "phase_ms": {k: v / 3 for k, v in phases.items()},
        "launches_per_substep": launches,
        "scaling": "strong",
        "sharding": f"{world} ranks, tanks by greedy particle balance" if world > 1 else "one GPU",
        "rank0_tanks": len(shard.tanks), "rank0_particles": shard.particles,
    }
    shard.close()
    return out


def surface_leg(device: int, reps: int = 10) -> list:
    """The fluid surface (buildFluidField + marchFluidField) per frame: the
    reference's published CPU case (8,192 particles at 40^3 and 64^3 samples,
    iso 0.5) and the 1M dam break at 128^3 and 256^3. GPU time is wall time of
    the C-ABI calls (field launch, march with its count read-back) after a
    synchronize. Its CPU baseline is the oracle port (field on all host
    cores, march serial as the reference's vertex order needs)."""
    import torch

    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu
    from oracle.bind import Oracle

    oracle = Oracle()
    threads = oracle.hardware_threads
    scene = W.reference_test_scene(8192, W.cell_count_for(8192))
    big = W.dam_break_1m()
    cases = [("reference_scene_8192", scene, 8192, None, 40), ("reference_scene_8192", scene, 8192, None, 64),
             ("dam_break_1m", big.params, big.count, big, 128), ("dam_break_1m", big.params, big.count, big, 256)]
    out = []
    for name, params, n, case, resolution in cases:
        with FluidSolverGpu(params, n, device=device) as solver:
            if case is None:
                solver.emit(params, n)
                for _ in range(60):
                    solver.step(params, 1.0 / 60.0)
            else:
                solver.upload(*case.initial_state())
                solver.run(case.dt, 2)
            solver.synchronize()
            solver.surface(resolution)  # warm-up (allocations, table upload)
            torch.cuda.synchronize(device)
            t0 = time.perf_counter()
            for _ in range(reps):
                solver.surface_field(resolution)
                written = solver.surface_march(0.5, 4_000_000)
            solver.synchronize()
            gpu_ms = (time.perf_counter() - t0) / reps * 1e3
            pos = solver.particles()
        origin = np.array(params.container_min[:3], np.float32)
        cell = ((np.array(params.container_max[:3], np.float32) - origin) / np.float32(resolution)).astype(np.float32)
        t0 = time.perf_counter()
        field = oracle.surface_field(params, pos, resolution, threads=threads)
        t1 = time.perf_counter()
        verts = oracle.march_field(field, resolution, origin, cell, 0.5, 4_000_000)
        t2 = time.perf_counter()
        del verts
        out.append({"workload": name, "particles": n, "resolution": resolution, "iso": 0.5, "vertices": written,
                    "gpu_ms_per_frame": gpu_ms,
                    "cpu_baseline": {"kind": "port", "ms_per_frame": (t2 - t0) * 1e3, "field_ms": (t1 - t0) * 1e3,
                                     "march_ms": (t2 - t1) * 1e3, "cores_field": threads, "cores_march": 1}})
    return out


def sustained_leg(steps: int, flush, device: int) -> dict:
    """The 1M dam break run for `steps` substeps from its initial state (the
    configuration's full length), each substep timed with CUDA events after an
    L2 flush. The dam collapses and compresses as it runs, so later substeps
    see more pairs per particle than the first ones: this is the figure a
    whole run gets."""
    import torch

    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

    case = W.dam_break_1m()
    n = case.count
    with FluidSolverGpu(case.params, n, device=device) as solver:
        solver.upload(*case.initial_state())
        stream = torch.cuda.ExternalStream(solver.stream(), device=torch.device("cuda", device))
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                starts[k].record(stream)
            solver.run(case.dt, 1)
            ends[k].record(stream)
        torch.cuda.synchronize()
        ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
        stats = solver.stats()
    mean = sum(ms) / steps
    tenth = max(1, steps // 10)
    return {
        "workload": case.name, "substeps": steps, "ms_per_step": mean, "value": n * case.dt / (mean / 1e3),
        "unit": UNIT, "ms_per_step_by_tenth": [sum(ms[i:i + tenth]) / len(ms[i:i + tenth])
                                               for i in range(0, steps, tenth)],
        "final_pairs_per_particle": stats.pairs_in_range / n, "final_mean_compression": stats.mean_compression,
        "l2": "flushed before every substep",
    }


def obstacles_leg(steps: int, flush, device: int, cpu: bool) -> dict:
    """The 1M dam break with five shape colliders and three force fields
    (workloads.obstacle_course_1m) beside the same tank without them: the
    first `steps` substeps of each from the initial state, each timed with
    CUDA events after an L2 flush. Its CPU baseline is the oracle with the
    same shapes, two substeps on all host cores."""
    import torch

    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

    # The shapes change the physics as well as adding two passes: particles
    # pressed against the colliders have more neighbours, which the density
    # and integrate phases pay for; the per-phase split and the final pair
    # count of each run show which is which.
    def timed(case) -> tuple[float, dict, float]:
        with FluidSolverGpu(case.params, case.count, device=device) as solver:
            solver.upload(*case.initial_state())
            solver.run(case.dt, 3)
            solver.synchronize()
            stream = torch.cuda.ExternalStream(solver.stream(), device=torch.device("cuda", device))
            total = 0.0
            for _ in range(steps):
                start = torch.cuda.Event(enable_timing=True)
                end = torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    flush.zero_()
                    start.record(stream)
                solver.run(case.dt, 1)
                end.record(stream)
                end.synchronize()
                total += start.elapsed_time(end)
            # Per-phase device times over a few more substeps (one by one).
            phases = {name: 0.0 for name in FluidSolverGpu.PROFILE_PHASES}
            for _ in range(5):
                with torch.cuda.stream(stream):
                    flush.zero_()
                for name, t in solver.profile(case.dt, 1).items():
                    phases[name] += t / 5
            pairs = solver.stats().pairs_in_range / case.count
        return total / steps, phases, pairs

    shapes = W.obstacle_course_1m()
    plain_ms, plain_phases, plain_pairs = timed(W.dam_break_1m())
    ms, phases, pairs = timed(shapes)
    n = shapes.count
    out = {
        "workload": shapes.name, "colliders": int(shapes.params.collider_count),
        "force_fields": int(shapes.params.field_count), "substeps": steps, "ms_per_step": ms,
        "value": n * shapes.dt / (ms / 1e3), "unit": UNIT, "plain_ms_per_step": plain_ms,
        "shape_overhead_ms": ms - plain_ms, "phase_ms": phases, "plain_phase_ms": plain_phases,
        "final_pairs_per_particle": pairs, "plain_final_pairs_per_particle": plain_pairs,
        "l2": "flushed before every substep",
    }
    if cpu:
        from oracle.bind import Oracle

        oracle = Oracle()
        pos, vel = shapes.initial_state()
        start = time.perf_counter()
        oracle.run_substeps(shapes.params, pos, vel, shapes.dt, 2, threads=oracle.hardware_threads)
        wall = time.perf_counter() - start
        out["cpu_baseline"] = {"kind": "port", "cores": oracle.hardware_threads, "ms_per_step": 1e3 * wall / 2,
                               "value": n * shapes.dt * 2 / wall, "unit": UNIT,
                               "sample": "2 whole-tank substeps with the same colliders and fields"}
    return out


def instances_leg(reps: int, flush, device: int, cpu: bool) -> dict:
    """The instance writer (sph_write_instances: one 224-byte draw instance
    and one 64-byte TLAS record per particle, then keepRendered) for the 1M
    dam break, timed with CUDA events after an L2 flush, against the measured
    HBM copy bandwidth: it reads 32 bytes a particle (position, previous
    position) and writes 288, plus keepRendered's 16 (the writer copies the
    position over the previous one in the same pass). Its CPU baseline is
    the oracle's restatement of the reference's CPU writer on all host
    cores."""
    import numpy as np
    import torch

    from computer_graphics_lab_00_gb300 import abi
    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

    case = W.dam_break_1m()
    n = case.count
    per_particle = 32 + abi.INSTANCE.itemsize + abi.TLAS_INSTANCE.itemsize + 16
    with FluidSolverGpu(case.params, n, device=device) as solver:
        solver.upload(*case.initial_state())
        solver.run(case.dt, 1)
        inst = torch.empty(n * abi.INSTANCE.itemsize, dtype=torch.uint8, device=f"cuda:{device}")
        tlas = torch.empty(n * abi.TLAS_INSTANCE.itemsize, dtype=torch.uint8, device=f"cuda:{device}")
        stream = torch.cuda.ExternalStream(solver.stream(), device=torch.device("cuda", device))

        def write():
            solver.write_instances(inst.data_ptr(), 0, 0, tlas.data_ptr(), 0, 0x1000, 0, abi.SPH_INSTANCES_WRITE_TLAS)

        for _ in range(3):
            write()
        solver.synchronize()
        total = 0.0
        for _ in range(reps):
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                flush.zero_()
                start.record(stream)
            write()
            end.record(stream)
            end.synchronize()
            total += start.elapsed_time(end)
        pos = solver.particles()
        prev = solver.previous_particles()
    ms = total / reps
    peak, peak_kind = measured_hbm_peak()
    achieved = per_particle * n / (ms / 1e3) / 1e9
    out = {
        "workload": case.name, "particles": n, "reps": reps, "ms_per_call": ms,
        "bytes_per_particle": per_particle,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "l2": "flushed before every call",
    }
    if cpu:
        from oracle.bind import Oracle

        oracle = Oracle()
        host_inst = np.zeros(n, abi.INSTANCE)
        host_tlas = np.zeros(n, abi.TLAS_INSTANCE)
        radius = float(case.params.container_min[3])
        start = time.perf_counter()
        oracle.write_instances(pos, prev, radius, host_inst, 0, 0, host_tlas, 0, 0x1000, 0,
                               abi.SPH_INSTANCES_WRITE_TLAS, threads=oracle.hardware_threads)
        wall = time.perf_counter() - start
        out["cpu_baseline"] = {"kind": "port", "cores": oracle.hardware_threads, "ms_per_call": 1e3 * wall,
                               "sample": "one call over the whole 1M tank"}
    return out


def learned_leg(steps: int, flush, device: int, plain_ms: float) -> dict:
    """The learned 5x-dt form on the same 1,048,576-particle tank: coarse
    steps of 1/240 s (plain force + tensor-core MLP correction), timed like
    the plain leg; accuracy against the plain fine run (1/1200 s) over 0.1 s."""
    import torch

    from computer_graphics_lab_00_gb300 import training as T
    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    case = W.dam_break_1m()
    n = case.count
    mlp = MlpGpu(device=device)
    T.load_model(mlp, WEIGHTS)
    pos, vel = case.initial_state()
    solver = FluidSolverGpu(case.params, n, device=device)
    solver.upload(pos, vel)
    stream = torch.cuda.ExternalStream(solver.stream(), device=torch.device("cuda", device))
    solver.run_learned(T.COARSE_DT, 3, mlp)
    solver.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            starts[k].record(stream)
        solver.run_learned(T.COARSE_DT, 1, mlp)
        ends[k].record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends)) / steps
    # Accuracy over 2 s from the initial state (checks every 0.1 s) against
    # the plain fine run, beside the plain coarse step without the network.
    fine = FluidSolverGpu(case.params, n, device=device)
    plain = FluidSolverGpu(case.params, n, device=device)
    for s in (fine, plain, solver):
        s.upload(pos, vel)
    err = {"learned": [], "plain": []}
    drift = {"learned": [], "plain": []}
    for _ in range(20):
        fine.run(T.FINE_DT, 120)
        solver.run_learned(T.COARSE_DT, 24, mlp)
        plain.run_learned(T.COARSE_DT, 24, None)
        sf = fine.stats()
        for name, s in (("learned", solver), ("plain", plain)):
            st = s.stats()
            err[name].append(abs(st.mean_compression - sf.mean_compression))
            drift[name].append(float(np.linalg.norm(np.array(st.centre_of_mass[:]) - np.array(sf.centre_of_mass[:]))))
    value = n * T.COARSE_DT / (ms / 1e3)
    plain_fine_value = n * T.FINE_DT / (plain_ms / 1e3)
    out = {
        "dt": T.COARSE_DT, "steps": steps, "ms_per_step": ms, "value": value, "unit": UNIT,
        "speedup_vs_plain_fine_step": value / plain_fine_value,
        "speedup_vs_plain_1_600": value / (n * case.dt / (plain_ms / 1e3)),
        "density_error_2s": {k: float(np.mean(v)) for k, v in err.items()},
        "com_drift_2s_m": {k: float(np.mean(v)) for k, v in drift.items()},
        "weights": str(WEIGHTS.relative_to(ROOT)),
    }
    for s in (solver, fine, plain, mlp):
        s.close()
    return out


def learned_eval_leg(device: int) -> dict:
    """Config 4's evaluation: 64 held-out dam-break/drop tanks of 32,768
    particles over 2 s; mean density error and centre-of-mass drift of the
    learned coarse step and of the plain coarse step (1/240 s) against the
    plain fine run (1/1200 s)."""
    from computer_graphics_lab_00_gb300 import training as T
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    held = T.learned_tanks(64, 32768, seed=T.HELD_OUT_SEED)
    with MlpGpu(device=device) as mlp:
        T.load_model(mlp, WEIGHTS)
        start = time.perf_counter()
        cmp = T.compare_with_fine(held, mlp, duration=2.0, every=0.1, device=device)
        wall = time.perf_counter() - start
    keep = ("mean_density_error", "final_density_error", "mean_com_drift_m", "final_com_drift_m")
    return {"tanks": 64, "particles_per_tank": 32768, "seconds": 2.0, "wall_s": wall,
            **{k: {q: v[q] for q in keep} for k, v in cmp.items()},
            "ratio_density": cmp["learned"]["mean_density_error"] / cmp["plain"]["mean_density_error"],
            "ratio_com": cmp["learned"]["mean_com_drift_m"] / cmp["plain"]["mean_com_drift_m"]}


def learned_batched_leg(coarse_steps: int, device: int) -> dict:
    """Config 5: 1,024 tanks of 8,192 particles (uneven blocks), learned
    coarse steps of 1/240 s with the fine solver as checker and per-tank
    fallback, against the plain batched form at the fine step (1/1200 s)
    over the same simulated time on the same GPU."""
    from computer_graphics_lab_00_gb300 import training as T
    from computer_graphics_lab_00_gb300.learned import MlpGpu

    tankset = T.learned_tanks(1024, 8192, seed=7)
    with MlpGpu(device=device) as mlp:
        T.load_model(mlp, WEIGHTS)
        learned = T.run_with_fallback(tankset, mlp, coarse_steps=coarse_steps, device=device)
    plain = T.run_plain_fine(tankset, coarse_steps=coarse_steps, device=device)
    errors = T.fallback_errors(learned, plain)
    return {"tanks": 1024, "particles_per_tank": 8192, "coarse_steps": coarse_steps,
            "speedup_vs_plain_fine": learned["sim_s_particles_per_s"] / plain["sim_s_particles_per_s"],
            "learned_value": learned["sim_s_particles_per_s"], "plain_fine_value": plain["sim_s_particles_per_s"],
            "unit": UNIT, "learned_wall_s": learned["wall_s"], "plain_fine_wall_s": plain["wall_s"],
            "vs_plain_fine": errors, "fallback_fraction": learned["fallback_fraction"],
            "judged_tank_intervals": learned["judged_tank_intervals"], "rejected": learned["rejected_checks"],
            "drift_fallbacks": learned["drift_fallbacks"], "check_errors_mean": learned["check_errors_mean"]}


def run_reference(args) -> None:
    """The reference's CPU solver path (oracle port, all host threads)."""
    from computer_graphics_lab_00_gb300 import workloads as W

    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle.bind import Oracle

    case = W.dam_break_1m()
    oracle = Oracle()
    threads = oracle.hardware_threads
    pos, vel = case.initial_state()
    for _ in range(max(args.warmup, 0)):
        t0 = time.perf_counter()
        pos, vel = oracle.substep(case.params, pos, vel, case.dt, threads=threads)
        last = time.perf_counter() - t0
    # Keep the whole run within a few minutes: cap the timed substeps.
    steps = args.steps
    budget = 150.0
    per = last if args.warmup > 0 else 1.0
    timed = max(1, min(steps, int(budget / max(per, 1e-3))))
    start = time.perf_counter()
    for _ in range(timed):
        pos, vel = oracle.substep(case.params, pos, vel, case.dt, threads=threads)
    wall = time.perf_counter() - start
    value = case.count * case.dt * timed / wall
    sample = (f"{timed} whole-tank substeps of the {case.count}-particle tank"
              + ("" if timed == steps else f" (of {steps} requested; capped to ~{budget:.0f} s)"))
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": timed, "warmup": args.warmup,
        "ms_per_step": 1e3 * wall / timed, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic", "config": workload_config(case, 1), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(out), flush=True)


def run_gb300(args) -> None:
    import torch

    from computer_graphics_lab_00_gb300 import workloads as W
    from computer_graphics_lab_00_gb300.fluid import FluidSolverGpu

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    case = W.dam_break_1m()
    n = case.count
    dt = case.dt
    pos0, vel0 = case.initial_state()
    solver = FluidSolverGpu(case.params, n, device=local)
    if args.neighbour_kernel is not None:
        solver.set_tuning(neighbour_kernel=args.neighbour_kernel)
    solver.upload(pos0, vel0)
    pairs = solver.stats()  # candidate and in-range pair counts of the initial state
    stream = torch.cuda.ExternalStream(solver.stream(), device=torch.device("cuda", local))
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()
        torch.cuda.synchronize()

    # Warm-up (builds the CUDA graph).
    warm = max(args.warmup, 3)
    solver.run(dt, warm)
    solver.synchronize()

    # Timed leg: device-resident state, one substep per timed interval. The
    # timed substeps are spread evenly over the workload's whole run (1,000
    # substeps: the dam collapses and compresses, and the cost per substep
    # changes with it), untimed substeps between them.
    gap = max(0, (case.steps - warm) // max(args.steps, 1) - 1)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    sampler = ClockSampler(local) if rank == 0 else None
    if sampler:
        sampler.__enter__()
    barrier()
    wall0 = time.perf_counter()
    pair_samples = []
    launches = 0  # our kernels inside the timed intervals (the substep graph, order remakes)
    for k in range(args.steps):
        if gap:
            solver.run(dt, gap)
        with torch.cuda.stream(stream):
            flush.zero_()
            starts[k].record(stream)
        before = solver.kernels_launched()
        solver.run(dt, 1)
        launches += solver.kernels_launched() - before
        ends[k].record(stream)
        if gap:
            # Candidate and in-range pair counts of the state just timed
            # (a counting pass outside the timed interval).
            st = solver.stats()
            pair_samples.append((st.candidates, st.pairs_in_range))
    barrier()
    wall = time.perf_counter() - wall0
    if sampler:
        sampler.__exit__(None, None, None)
    device_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))

    # Per-phase device times (same kernels, launched one by one between events).
    phases = {name: 0.0 for name in FluidSolverGpu.PROFILE_PHASES}
    prof_steps = min(args.steps, 50)
    for _ in range(prof_steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        for name, ms in solver.profile(dt, 1).items():
            phases[name] += ms
    phases = {k: v / prof_steps for k, v in phases.items()}

    # End-to-end leg: host state in pinned memory, copies inside the timed
    # region. Each step is one sph_step_host call: upload the state (32 B a
    # particle), one substep, download it (32 B a particle), the velocity
    # upload overlapping the keys and sort.
    e2e_steps = args.e2e_steps or min(args.steps, 100)
    # From the state the timed leg ended in.
    end_pos, end_vel = solver.state()
    host_pos = torch.from_numpy(end_pos.copy()).pin_memory()
    host_vel = torch.from_numpy(end_vel.copy()).pin_memory()
    hp, hv = host_pos.data_ptr(), host_vel.data_ptr()
    solver.step_host(hp, hv, n, dt, 1, hp, hv)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        solver.step_host(hp, hv, n, dt, 1, hp, hv)
    barrier()
    e2e_wall = time.perf_counter() - t0

    # Max over ranks.
    times = torch.tensor([device_ms, e2e_wall], dtype=torch.float64, device=f"cuda:{local}")
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(times, op=dist.ReduceOp.MAX)
    device_ms, e2e_wall = float(times[0]), float(times[1])
    batched = batched_leg(args.batched_steps, flush, local, world) if args.batched_steps > 0 else None
    if rank != 0:
        solver.close()
        return

    total_particles = n * world
    value = total_particles * dt * args.steps / (device_ms / 1e3)
    e2e_value = total_particles * dt * e2e_steps / e2e_wall

    # Roofline of the dominant kernel: algorithmic bytes per launch.
    cells = int(case.params.lattice[3])
    alg_bytes = {
        "keys": 20 * n + 8 * cells,
        "sort": 16 * n + 20 * n * 2,
        "bounds_gather": 72 * n,
        "density": 24 * n,     # read own position 16 B, write rho + pressure 8 B
        "integrate": 64 * n,   # read own pos + vel 32 B, write pos + vel 32 B
    }
    dominant = max(phases, key=phases.get)
    peak, peak_kind = measured_hbm_peak()
    achieved = alg_bytes[dominant] / (phases[dominant] / 1e3) / 1e9
    traffic = None
    traffic_file = ROOT / "profiles" / "traffic_per_launch.json"
    if traffic_file.exists():
        try:
            traffic = json.loads(traffic_file.read_text()).get(dominant)
        except Exception:
            traffic = None
    step_alg = 120 * n + 12 * cells
    step_ms = device_ms / args.steps
    if pair_samples:
        cand = sum(c for c, _ in pair_samples) / len(pair_samples)
        inr = sum(r for _, r in pair_samples) / len(pair_samples)
    else:
        cand, inr = pairs.candidates, pairs.pairs_in_range
    flops = 20 * cand + 55 * inr
    # Nominal FP32 rate of this device: SMs x 128 lanes x 2 flop (FMA) x the
    # maximum SM clock (read from the device; MEASURED_PEAKS.json's if absent).
    props = torch.cuda.get_device_properties(local)
    sm_count = props.multi_processor_count
    max_mhz = None
    try:
        max_mhz = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("sm_max_mhz"))
    except Exception:
        pass
    if clocks_max := (sampler.summary().get("sm_max_mhz") if sampler else None):
        max_mhz = float(clocks_max)
    if not max_mhz:
        max_mhz = 2070.0
    nominal_fp32 = sm_count * 128 * 2 * max_mhz * 1e6 / 1e12

    clocks = sampler.summary() if sampler else None
    out = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": max(args.warmup, 3),
        "ms_per_step": step_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {**workload_config(case, world), "neighbour_kernel": solver.tuning()["neighbour_kernel"],
                   "grid_sort": solver.tuning()["sort"]},
        "particle_steps_per_s": total_particles * args.steps / (device_ms / 1e3),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 32 * n, "d2h_bytes_per_step": 32 * n,
                "steps": e2e_steps, "ms_per_step": 1e3 * e2e_wall / e2e_steps},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs", "traffic": traffic,
                     "alg_bytes_per_launch": alg_bytes[dominant]},
        "step_roofline": {"alg_bytes": step_alg, "achieved_gbs": step_alg / (step_ms / 1e3) / 1e9,
                          "frac_of_peak": step_alg / (step_ms / 1e3) / 1e9 / peak},
        "fp32": {"alg_flops_per_step": flops, "achieved_tflops": flops / (step_ms / 1e3) / 1e12,
                 "nominal_peak_tflops": nominal_fp32, "frac": flops / (step_ms / 1e3) / 1e12 / nominal_fp32,
                 "sm_count": sm_count, "sm_max_mhz": max_mhz, "candidates": cand, "pairs_in_range": inr,
                 "pairs_from": "mean over the timed substeps" if pair_samples else "initial state"},
        "phase_ms": phases,
        "gpu_launches": launches,
        "clocks": clocks,
        "wall_s_timed": wall,
    }
    if world == 1 and args.sustained_steps > 0:
        out["sustained"] = sustained_leg(args.sustained_steps, flush, local)
    if world == 1 and args.obstacle_steps > 0:
        out["obstacles"] = obstacles_leg(args.obstacle_steps, flush, local, not args.no_cpu_baseline)
    if world == 1 and args.instance_reps > 0:
        out["instances"] = instances_leg(args.instance_reps, flush, local, not args.no_cpu_baseline)
    if world == 1 and args.surface:
        out["surface"] = surface_leg(local)
    if world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(case, args.cpu_seconds)
    solver.close()
    # The batched and learned legs go last: they close the JSON line.
    if batched is not None:
        out["batched"] = batched
    if world == 1 and WEIGHTS.exists():
        if args.learned_steps > 0:
            out["learned"] = learned_leg(args.learned_steps, flush, local, step_ms)
        if args.learned_eval:
            out["learned_eval"] = learned_eval_leg(local)
        if args.fallback_steps > 0:
            out["learned_batched"] = learned_batched_leg(args.fallback_steps, local)
    print(json.dumps(out), flush=True)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
