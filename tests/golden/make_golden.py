"""Generates the golden vectors in tests/golden/ from the reference itself.

The reference's unmodified src/physics/fluid_sph.cpp is compiled in place
(oracle/ref/Makefile -> oracle/_ref/libsph_ref.so) and run on small seeded
cases; its outputs are frozen here so that machines without the reference
tree (the GPU host) can still pin the oracle and the CUDA path to it.

    python tests/golden/make_golden.py              # the small cases (.npz)
    python tests/golden/make_golden.py --long-run   # the 1M-particle, 1,000-substep digests (.json)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from computer_graphics_lab_00_gb300 import workloads as W  # noqa: E402
from oracle.bind import Reference, build_reference  # noqa: E402

OUT = Path(__file__).resolve().parent


def params_bytes(params) -> np.ndarray:
    return np.frombuffer(bytes(params), dtype=np.uint8).copy()


def compact_slots(counts: np.ndarray, slots: np.ndarray) -> np.ndarray:
    filled = np.minimum(counts, 32)
    used = (np.arange(32)[None, :] < filled[:, None]).reshape(-1)
    return slots[used]


def scene_frames() -> dict:
    """tests/fluid_test.cpp's scene: emit 1024, then 30 frames of 1/60 s."""
    params = W.reference_test_scene(1024)
    ref = Reference()
    ref.emit(params, 1024)
    emit_pos, emit_vel = ref.state()
    ref.step(params, 1.0 / 60.0, frames=30)
    pos, vel = ref.state()
    return {"params": params_bytes(params), "emit_pos": emit_pos, "emit_vel": emit_vel, "pos_30": pos, "vel_30": vel}


def dam_break_small() -> dict:
    """2,048 jittered particles (16 x 16 x 8) in a 0.6 m box, 4,096 buckets."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(0.6, 0.6, 0.6), lattice=(16, 16, 8),
                           cell_count=4096)
    pos, vel = W.jittered_block(params, 2048, seed=11)
    ref = Reference()
    cell_of, counts, slots = ref.grid_build(params, pos)
    ref.set_state(pos, vel)
    ref.substep(params, 1.0 / 600.0)
    pos1, vel1 = ref.state()
    for _ in range(19):
        ref.substep(params, 1.0 / 600.0)
    pos20, vel20 = ref.state()
    return {"params": params_bytes(params), "pos": pos, "vel": vel, "cell_of": cell_of, "cell_counts": counts,
            "cell_slots": compact_slots(counts, slots), "pos_1": pos1, "vel_1": vel1, "pos_20": pos20,
            "vel_20": vel20}


def collisions_overflow() -> dict:
    """1,024 particles with 1,024 buckets (colliding neighbour cells), 200 of
    them packed into one cell (an overflowing bucket)."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(0.5, 0.5, 0.5), lattice=(8, 8, 16),
                           cell_count=1024)
    pos, vel = W.jittered_block(params, 1024, seed=21)
    u = W.uniform01(99, np.arange(600, dtype=np.uint64)).reshape(200, 3)
    pos[:200, :3] = np.float32(0.2) + u * np.float32(0.039)
    ref = Reference()
    cell_of, counts, slots = ref.grid_build(params, pos)
    ref.set_state(pos, vel)
    for _ in range(5):
        ref.substep(params, 1.0 / 600.0)
    pos5, vel5 = ref.state()
    return {"params": params_bytes(params), "pos": pos, "vel": vel, "cell_of": cell_of, "cell_counts": counts,
            "cell_slots": compact_slots(counts, slots), "pos_5": pos5, "vel_5": vel5}


def obstacles_small() -> dict:
    """2,048 particles with one collider of every shape and one field of
    every kind (workloads.obstacles_small), 1 and 40 substeps."""
    params = W.obstacles_small()
    pos, vel = W.jittered_block(params, 2048, seed=13)
    ref = Reference()
    ref.set_state(pos, vel)
    ref.substep(params, 1.0 / 600.0)
    pos1, vel1 = ref.state()
    for _ in range(39):
        ref.substep(params, 1.0 / 600.0)
    pos40, vel40 = ref.state()
    return {"params": params_bytes(params), "pos": pos, "vel": vel, "pos_1": pos1, "vel_1": vel1, "pos_40": pos40,
            "vel_40": vel40}


def surface_small() -> dict:
    """The reference's marching-cubes table, and buildFluidField /
    marchFluidField (serial) on dam_break_small after 20 substeps, resolution
    24, iso 0.5: all vertices, and the prefix a 600-vertex capacity keeps."""
    params = W.make_params(container_min=(0.0, 0.0, 0.0), container_max=(0.6, 0.6, 0.6), lattice=(16, 16, 8),
                           cell_count=4096)
    pos, vel = W.jittered_block(params, 2048, seed=11)
    ref = Reference()
    ref.set_state(pos, vel)
    for _ in range(20):
        ref.substep(params, 1.0 / 600.0)
    pos20, _ = ref.state()
    field = ref.surface_field(params, pos20, 24)
    origin = np.array(params.container_min[:3], np.float32)
    cell = ((np.array(params.container_max[:3], np.float32) - origin) / np.float32(24)).astype(np.float32)
    full = ref.march_field(field, 24, origin, cell, 0.5, 200000)
    short = ref.march_field(field, 24, origin, cell, 0.5, 600)
    return {"params": params_bytes(params), "mc_table": ref.mc_table(), "pos": pos20, "field_24": field,
            "vertices_24": full.view(np.uint8).reshape(-1, 16), "vertices_24_cap600": short.view(np.uint8).reshape(-1, 16)}


def state_digest(pos: np.ndarray, vel: np.ndarray) -> tuple[str, str]:
    """SHA-256 of the float32 position and velocity arrays (id order)."""
    import hashlib

    return (hashlib.sha256(np.ascontiguousarray(pos, np.float32).tobytes()).hexdigest(),
            hashlib.sha256(np.ascontiguousarray(vel, np.float32).tobytes()).hexdigest())


def long_run_1m(threads: int) -> dict:
    """The 1,048,576-particle dam break (dam_break_1m) over its 1,000 substeps
    of 1/600 s through the reference: every 100 substeps the digests of the
    whole state and its FP64 mean density and centre of mass."""
    case = W.dam_break_1m()
    pos, vel = case.initial_state()
    ref = Reference()
    ref.set_state(pos, vel)
    rows = []
    for k in range(1, case.steps + 1):
        ref.substep(case.params, case.dt, threads=threads)
        if k % 100 == 0:
            pos, vel = ref.state()
            dp, dv = state_digest(pos, vel)
            p64 = pos.astype(np.float64)
            rows.append({"substep": k, "pos_sha256": dp, "vel_sha256": dv, "mean_density": float(p64[:, 3].mean()),
                         "centre_of_mass": [float(p64[:, a].mean()) for a in range(3)]})
            print(rows[-1], flush=True)
    return {"workload": case.name, "particles": case.count, "dt": case.dt, "checkpoints": rows}


def main() -> None:
    if build_reference() is None:
        raise SystemExit("the reference tree is needed to regenerate the golden vectors")
    if "--long-run" in sys.argv:
        # About ten minutes on 8 cores; kept out of the default regeneration.
        import json
        import os

        data = long_run_1m(os.cpu_count() or 1)
        (OUT / "dam_break_1m_long.json").write_text(json.dumps(data, indent=1))
        return
    for name, make in (("scene_frames", scene_frames), ("dam_break_small", dam_break_small),
                       ("collisions_overflow", collisions_overflow), ("obstacles_small", obstacles_small),
                       ("surface_small", surface_small)):
        data = make()
        np.savez_compressed(OUT / f"{name}.npz", **data)
        print(name, {k: v.shape for k, v in data.items()})


if __name__ == "__main__":
    main()
