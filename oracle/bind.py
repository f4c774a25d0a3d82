"""ctypes bindings of the CPU oracle and of the reference checker.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).

* `Oracle` wraps oracle/build/libsph_oracle.so, the restatement of the
  reference's CPU fluid path (oracle/sph_oracle.cpp).
* `Reference` wraps oracle/_ref/libsph_ref.so: the reference's own
  src/physics/fluid_sph.cpp compiled in place (oracle/ref/Makefile). It can
  only be built where the reference tree is present.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

from computer_graphics_lab_00_gb300.abi import SphFluidSettings, SphParams, SphStats

ORACLE_DIR = Path(__file__).resolve().parent
ORACLE_LIB = ORACLE_DIR / "build" / "libsph_oracle.so"
REFERENCE_LIB = ORACLE_DIR / "_ref" / "libsph_ref.so"
# The reference source tree; SPH_REFERENCE_TREE overrides the default location.
REFERENCE_TREE = Path(os.environ.get("SPH_REFERENCE_TREE", "/root/reference"))

P = ctypes.POINTER
f32p = P(ctypes.c_float)
u32p = P(ctypes.c_uint32)
u64p = P(ctypes.c_uint64)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(f32p)


def _up(a: np.ndarray):
    return a.ctypes.data_as(u32p)


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
    return ORACLE_LIB


def build_reference() -> Path | None:
    """Compiles the reference checker when the reference tree is present."""
    if not (REFERENCE_TREE / "src" / "physics" / "fluid_sph.cpp").exists():
        return None
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR / "ref"), f"REFERENCE={REFERENCE_TREE}"], check=True)
    return REFERENCE_LIB


def _as_state(pos: np.ndarray, vel: np.ndarray | None):
    pos = np.ascontiguousarray(pos, dtype=np.float32).copy()
    n = pos.shape[0]
    vel = np.zeros((n, 4), np.float32) if vel is None else np.ascontiguousarray(vel, dtype=np.float32).copy()
    return pos, vel


def _march(fn, field, resolution, origin, cell, iso, capacity):
    from computer_graphics_lab_00_gb300.abi import SURFACE_VERTEX

    field = np.ascontiguousarray(field, dtype=np.float32)
    o = np.asarray(origin, np.float32)
    c = np.asarray(cell, np.float32)
    out = np.zeros(max(capacity, 1), SURFACE_VERTEX)
    written = ctypes.c_uint32()
    rc = fn(_fp(field), resolution, _fp(o), _fp(c), ctypes.c_float(iso), out.ctypes.data, capacity,
            ctypes.byref(written))
    assert rc == 0
    return out[: written.value].copy()


class Oracle:
    """The restated CPU solver. Every call copies its inputs."""

    _lib = None

    def __init__(self):
        if Oracle._lib is None:
            if not ORACLE_LIB.exists():
                build_oracle()
            lib = ctypes.CDLL(str(ORACLE_LIB))
            lib.oracle_abi.restype = ctypes.c_int
            lib.oracle_spatial_hash.restype = ctypes.c_uint32
            lib.oracle_spatial_hash.argtypes = [ctypes.c_int32] * 3 + [ctypes.c_uint32]
            lib.oracle_spatial_cell.argtypes = [f32p, ctypes.c_float, P(ctypes.c_int32)]
            lib.oracle_derive_params.argtypes = [P(SphFluidSettings), f32p, ctypes.c_uint32, ctypes.c_uint32, P(SphParams)]
            lib.oracle_fluid_substeps.restype = ctypes.c_uint32
            lib.oracle_fluid_substeps.argtypes = [P(SphParams), ctypes.c_float]
            lib.oracle_emit.argtypes = [P(SphParams), ctypes.c_uint32, f32p, f32p]
            lib.oracle_grid_build.argtypes = [P(SphParams), f32p, ctypes.c_uint32, u32p, u32p, u32p, ctypes.c_uint32]
            lib.oracle_substep.argtypes = [P(SphParams), f32p, f32p, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint32]
            lib.oracle_step.argtypes = [P(SphParams), f32p, f32p, ctypes.c_uint32, ctypes.c_float, ctypes.c_uint32]
            lib.oracle_density.argtypes = [P(SphParams), f32p, f32p, ctypes.c_uint32, ctypes.c_uint32]
            lib.oracle_pair_counts.argtypes = [P(SphParams), f32p, ctypes.c_uint32, u64p, u64p, ctypes.c_uint32]
            lib.oracle_stats.argtypes = [P(SphParams), f32p, f32p, ctypes.c_uint32, P(SphStats)]
            lib.oracle_hardware_threads.restype = ctypes.c_uint32
            lib.oracle_mc_table.argtypes = [ctypes.c_void_p]
            lib.oracle_surface_field.argtypes = [P(SphParams), f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                 f32p]
            lib.oracle_march_field.argtypes = [f32p, ctypes.c_uint32, f32p, f32p, ctypes.c_float, ctypes.c_void_p,
                                               ctypes.c_uint32, P(ctypes.c_uint32)]
            lib.oracle_write_instances.argtypes = [f32p, f32p, ctypes.c_uint32, ctypes.c_float, ctypes.c_void_p,
                                                   ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_uint32,
                                                   ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
            Oracle._lib = lib
        self.lib = Oracle._lib

    @property
    def hardware_threads(self) -> int:
        return int(self.lib.oracle_hardware_threads())

    def mc_table(self) -> np.ndarray:
        out = np.zeros((256, 16), np.int8)
        self.lib.oracle_mc_table(out.ctypes.data)
        return out

    def surface_field(self, params: SphParams, pos, resolution: int, threads: int = 1) -> np.ndarray:
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        samples = resolution + 1
        field = np.zeros(samples ** 3, np.float32)
        rc = self.lib.oracle_surface_field(ctypes.byref(params), _fp(pos), pos.shape[0], resolution, threads, _fp(field))
        assert rc == 0
        return field

    def march_field(self, field, resolution: int, origin, cell, iso: float, capacity: int):
        return _march(self.lib.oracle_march_field, field, resolution, origin, cell, iso, capacity)

    def write_instances(self, pos, prev, radius: float, instances, instance_base: int = 0, sphere_mesh: int = 0,
                        tlas=None, tlas_base: int = 0, blas: int = 0, fluid_index: int = 0, flags: int = 0,
                        threads: int = 1) -> None:
        """fluid.cpp:402-466 into the given structured arrays (abi.INSTANCE,
        abi.TLAS_INSTANCE), which must hold the bases plus the count."""
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        prev = np.ascontiguousarray(prev if prev is not None else pos, dtype=np.float32)
        rc = self.lib.oracle_write_instances(
            _fp(pos), _fp(prev), pos.shape[0], ctypes.c_float(radius), instances.ctypes.data, instance_base,
            sphere_mesh, None if tlas is None else tlas.ctypes.data, tlas_base, blas, fluid_index, flags, threads)
        assert rc == 0

    def spatial_hash(self, cx: int, cy: int, cz: int, cells: int) -> int:
        return int(self.lib.oracle_spatial_hash(cx, cy, cz, cells))

    def spatial_cell(self, p, h: float):
        pos = np.asarray(p, dtype=np.float32)
        out = (ctypes.c_int32 * 3)()
        self.lib.oracle_spatial_cell(_fp(pos), ctypes.c_float(h), out)
        return tuple(out)

    def derive_params(self, settings: SphFluidSettings, world, count: int, cells: int) -> SphParams:
        w = np.asarray(world, dtype=np.float32)
        out = SphParams()
        rc = self.lib.oracle_derive_params(ctypes.byref(settings), _fp(w), count, cells, ctypes.byref(out))
        assert rc == 0
        return out

    def fluid_substeps(self, params: SphParams, dt: float) -> int:
        return int(self.lib.oracle_fluid_substeps(ctypes.byref(params), ctypes.c_float(dt)))

    def emit(self, params: SphParams, count: int):
        pos = np.zeros((count, 4), np.float32)
        vel = np.zeros((count, 4), np.float32)
        self.lib.oracle_emit(ctypes.byref(params), count, _fp(pos), _fp(vel))
        return pos, vel

    def grid_build(self, params: SphParams, pos: np.ndarray, threads: int = 1):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        n = pos.shape[0]
        cells = params.lattice[3]
        cell_of = np.zeros(n, np.uint32)
        counts = np.zeros(cells, np.uint32)
        slots = np.full(cells * 32, 0xFFFFFFFF, np.uint32)
        rc = self.lib.oracle_grid_build(ctypes.byref(params), _fp(pos), n, _up(cell_of), _up(counts), _up(slots), threads)
        assert rc == 0
        return cell_of, counts, slots

    def substep(self, params: SphParams, pos, vel, dt: float, threads: int = 1):
        pos, vel = _as_state(pos, vel)
        rc = self.lib.oracle_substep(ctypes.byref(params), _fp(pos), _fp(vel), pos.shape[0], ctypes.c_float(dt), threads)
        assert rc == 0
        return pos, vel

    def step(self, params: SphParams, pos, vel, frame_dt: float, threads: int = 1, frames: int = 1):
        pos, vel = _as_state(pos, vel)
        for _ in range(frames):
            rc = self.lib.oracle_step(ctypes.byref(params), _fp(pos), _fp(vel), pos.shape[0], ctypes.c_float(frame_dt), threads)
            assert rc == 0
        return pos, vel

    def run_substeps(self, params: SphParams, pos, vel, dt: float, substeps: int, threads: int = 1):
        pos, vel = _as_state(pos, vel)
        for _ in range(substeps):
            rc = self.lib.oracle_substep(ctypes.byref(params), _fp(pos), _fp(vel), pos.shape[0], ctypes.c_float(dt), threads)
            assert rc == 0
        return pos, vel

    def density(self, params: SphParams, pos, vel, threads: int = 1):
        pos, vel = _as_state(pos, vel)
        rc = self.lib.oracle_density(ctypes.byref(params), _fp(pos), _fp(vel), pos.shape[0], threads)
        assert rc == 0
        return pos, vel

    def pair_counts(self, params: SphParams, pos, threads: int = 1):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        p = ctypes.c_uint64()
        q = ctypes.c_uint64()
        rc = self.lib.oracle_pair_counts(ctypes.byref(params), _fp(pos), pos.shape[0], ctypes.byref(p), ctypes.byref(q), threads)
        assert rc == 0
        return int(p.value), int(q.value)

    def stats(self, params: SphParams, pos, vel) -> SphStats:
        pos, vel = _as_state(pos, vel)
        out = SphStats()
        self.lib.oracle_stats(ctypes.byref(params), _fp(pos), _fp(vel), pos.shape[0], ctypes.byref(out))
        return out


class Reference:
    """The reference's own FluidSolver, compiled in place. One solver per object."""

    _lib = None

    @staticmethod
    def available() -> bool:
        return REFERENCE_LIB.exists()

    def __init__(self):
        if Reference._lib is None:
            lib = ctypes.CDLL(str(REFERENCE_LIB))
            lib.ref_solver_create.restype = ctypes.c_void_p
            lib.ref_solver_destroy.argtypes = [ctypes.c_void_p]
            lib.ref_solver_set_state.argtypes = [ctypes.c_void_p, f32p, f32p, ctypes.c_uint32]
            lib.ref_solver_get_state.argtypes = [ctypes.c_void_p, f32p, f32p]
            lib.ref_solver_get_previous.argtypes = [ctypes.c_void_p, f32p]
            lib.ref_solver_count.restype = ctypes.c_uint32
            lib.ref_solver_count.argtypes = [ctypes.c_void_p]
            lib.ref_solver_emit.argtypes = [ctypes.c_void_p, P(SphParams), ctypes.c_uint32]
            lib.ref_solver_step.argtypes = [ctypes.c_void_p, P(SphParams), ctypes.c_float, ctypes.c_uint32]
            lib.ref_solver_substep.argtypes = [ctypes.c_void_p, P(SphParams), ctypes.c_float, ctypes.c_uint32]
            lib.ref_solver_keep_rendered.argtypes = [ctypes.c_void_p]
            lib.ref_grid_build.argtypes = [P(SphParams), f32p, ctypes.c_uint32, u32p, u32p, u32p, ctypes.c_uint32]
            lib.ref_fluid_substeps.restype = ctypes.c_uint32
            lib.ref_fluid_substeps.argtypes = [P(SphParams), ctypes.c_float]
            lib.ref_derive_params.argtypes = [P(SphFluidSettings), f32p, ctypes.c_uint32, ctypes.c_uint32, P(SphParams)]
            lib.ref_mc_table.argtypes = [ctypes.c_void_p]
            lib.ref_surface_field.argtypes = [P(SphParams), f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                              f32p]
            lib.ref_march_field.argtypes = [f32p, ctypes.c_uint32, f32p, f32p, ctypes.c_float, ctypes.c_void_p,
                                            ctypes.c_uint32, P(ctypes.c_uint32)]
            Reference._lib = lib
        self.lib = Reference._lib
        self.handle = ctypes.c_void_p(self.lib.ref_solver_create())

    def __del__(self):
        if getattr(self, "handle", None) and self.lib is not None:
            self.lib.ref_solver_destroy(self.handle)
            self.handle = None

    def set_state(self, pos, vel=None):
        pos, vel = _as_state(pos, vel)
        self.lib.ref_solver_set_state(self.handle, _fp(pos), _fp(vel), pos.shape[0])

    def state(self):
        n = self.lib.ref_solver_count(self.handle)
        pos = np.zeros((n, 4), np.float32)
        vel = np.zeros((n, 4), np.float32)
        self.lib.ref_solver_get_state(self.handle, _fp(pos), _fp(vel))
        return pos, vel

    def previous(self):
        n = self.lib.ref_solver_count(self.handle)
        pos = np.zeros((n, 4), np.float32)
        self.lib.ref_solver_get_previous(self.handle, _fp(pos))
        return pos

    def emit(self, params: SphParams, count: int):
        self.lib.ref_solver_emit(self.handle, ctypes.byref(params), count)

    def step(self, params: SphParams, frame_dt: float, threads: int = 1, frames: int = 1):
        for _ in range(frames):
            self.lib.ref_solver_step(self.handle, ctypes.byref(params), ctypes.c_float(frame_dt), threads)

    def substep(self, params: SphParams, dt: float, threads: int = 1):
        self.lib.ref_solver_substep(self.handle, ctypes.byref(params), ctypes.c_float(dt), threads)

    def keep_rendered(self):
        self.lib.ref_solver_keep_rendered(self.handle)

    def grid_build(self, params: SphParams, pos: np.ndarray, threads: int = 1):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        n = pos.shape[0]
        cells = params.lattice[3]
        cell_of = np.zeros(n, np.uint32)
        counts = np.zeros(cells, np.uint32)
        slots = np.full(cells * 32, 0xFFFFFFFF, np.uint32)
        self.lib.ref_grid_build(ctypes.byref(params), _fp(pos), n, _up(cell_of), _up(counts), _up(slots), threads)
        return cell_of, counts, slots

    def fluid_substeps(self, params: SphParams, dt: float) -> int:
        return int(self.lib.ref_fluid_substeps(ctypes.byref(params), ctypes.c_float(dt)))

    def mc_table(self) -> np.ndarray:
        out = np.zeros((256, 16), np.int8)
        self.lib.ref_mc_table(out.ctypes.data)
        return out

    def surface_field(self, params: SphParams, pos, resolution: int, threads: int = 1) -> np.ndarray:
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        field = np.zeros((resolution + 1) ** 3, np.float32)
        self.lib.ref_surface_field(ctypes.byref(params), _fp(pos), pos.shape[0], resolution, threads, _fp(field))
        return field

    def march_field(self, field, resolution: int, origin, cell, iso: float, capacity: int):
        """marchFluidField without a job system: vertices in cell order."""
        return _march(self.lib.ref_march_field, field, resolution, origin, cell, iso, capacity)

    def derive_params(self, settings: SphFluidSettings, world, count: int, cells: int) -> SphParams:
        w = np.asarray(world, dtype=np.float32)
        out = SphParams()
        self.lib.ref_derive_params(ctypes.byref(settings), _fp(w), count, cells, ctypes.byref(out))
        return out
