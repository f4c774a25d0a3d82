"""Python mirror of the reference's fluid-solver API over the C ABI.

`FluidSolverGpu` keeps the method names and argument meaning of
`physics::FluidSolver` (src/physics/fluid_sph.h:101-127): `emit(params,
count)`, `step(params, delta_seconds)`, `particles()`,
`previous_particles()`, `keep_rendered()`, `particle_count()`. The solver
state lives on the GPU; host arrays are (N, 4) float32 in the reference's
AoS layout. Every call goes through libsph_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi
from .abi import SphFluidSettings, SphParams, SphStats, check, load


def _ptr(a: np.ndarray | None):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def derive_fluid_params(settings: SphFluidSettings, emitter_world, particle_count: int, cell_count: int) -> SphParams:
    """physics::deriveFluidParams (fluid_sph.cpp:65-100) without scene colliders or fields."""
    lib = load()
    world = np.ascontiguousarray(emitter_world, dtype=np.float32)
    out = SphParams()
    check(lib.sph_derive_params(ctypes.byref(settings), world.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                particle_count, cell_count, ctypes.byref(out)), "sph_derive_params")
    return out


def fluid_substeps(params: SphParams, delta_seconds: float) -> int:
    """physics::fluidSubsteps (fluid_sph.cpp:128-136)."""
    lib = load()
    out = ctypes.c_uint32()
    check(lib.sph_fluid_substeps(ctypes.byref(params), ctypes.c_float(delta_seconds), ctypes.byref(out)),
          "sph_fluid_substeps")
    return int(out.value)


def cell_count_for(particles: int) -> int:
    """gfx::cellCountFor (src/gfx/fluid.cpp:50-52)."""
    return int(load().sph_cell_count_for(particles))


def cell_count_uncapped(particles: int) -> int:
    return int(load().sph_cell_count_uncapped(particles))


def surface_table() -> np.ndarray:
    """The marching-cubes case table the device uses (256 x 16, -1 ends a case)."""
    out = np.zeros((256, abi.SPH_MC_TABLE_WIDTH), np.int8)
    check(load().sph_surface_table(out.ctypes.data), "sph_surface_table")
    return out


def march_field(field, resolution: int, origin, cell, iso: float, capacity: int, device: int = 0) -> np.ndarray:
    """physics::marchFluidField (marching_cubes.cpp:397-481) of a host field on
    the GPU; returns the vertices (structured array, abi.SURFACE_VERTEX)."""
    f = np.ascontiguousarray(field, dtype=np.float32)
    if f.size != (resolution + 1) ** 3:
        raise ValueError("field must hold (resolution + 1)^3 samples")
    o = np.ascontiguousarray(origin, dtype=np.float32)
    c = np.ascontiguousarray(cell, dtype=np.float32)
    out = np.zeros(max(capacity, 1), abi.SURFACE_VERTEX)
    written = ctypes.c_uint32()
    check(load().sph_march_field(f.ctypes.data, resolution, o.ctypes.data, c.ctypes.data, ctypes.c_float(iso),
                                 out.ctypes.data, capacity, ctypes.byref(written), device), "sph_march_field")
    return out[: written.value].copy()


class FluidSolverGpu:
    """One fluid on one GPU; the device twin of physics::FluidSolver."""

    def __init__(self, params: SphParams, capacity: int, device: int = 0):
        self._lib = load()
        self._ctx = ctypes.c_void_p()
        self._params = params.copy()
        check(self._lib.sph_create(ctypes.byref(self._params), capacity, device, ctypes.byref(self._ctx)),
              "sph_create")
        self.capacity = capacity

    # -- lifetime ---------------------------------------------------------
    def close(self) -> None:
        if self._ctx:
            self._lib.sph_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, status: int, what: str) -> None:
        check(status, what, self._ctx)

    def _use(self, params: SphParams | None) -> None:
        if params is not None and bytes(params) != bytes(self._params):
            self._check(self._lib.sph_set_params(self._ctx, ctypes.byref(params)), "sph_set_params")
            self._params = params.copy()

    # -- FluidSolver surface ---------------------------------------------------
    def emit(self, params: SphParams, count: int) -> None:
        self._use(params)
        self._check(self._lib.sph_emit(self._ctx, count), "sph_emit")

    def step(self, params: SphParams, delta_seconds: float) -> None:
        self._use(params)
        self._check(self._lib.sph_step(self._ctx, ctypes.c_float(delta_seconds)), "sph_step")

    def substep(self, dt: float) -> None:
        self._check(self._lib.sph_substep(self._ctx, ctypes.c_float(dt)), "sph_substep")

    def run(self, dt: float, substeps: int) -> None:
        """Enqueues substeps without waiting for them."""
        self._check(self._lib.sph_run(self._ctx, ctypes.c_float(dt), substeps), "sph_run")

    def run_learned(self, dt: float, substeps: int, mlp=None) -> None:
        """Learned coarse substeps (mlp None: zero correction, the plain bits)."""
        self._check(self._lib.sph_run_learned(self._ctx, ctypes.c_float(dt), substeps,
                                              None if mlp is None else mlp.handle), "sph_run_learned")

    def particle_count(self) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sph_particle_count(self._ctx, ctypes.byref(out)), "sph_particle_count")
        return int(out.value)

    def particles(self) -> np.ndarray:
        """(N, 4) float32: xyz position, w density."""
        pos = np.empty((self.particle_count(), 4), np.float32)
        self._check(self._lib.sph_download(self._ctx, _ptr(pos), None), "sph_download")
        return pos

    def velocities(self) -> np.ndarray:
        """(N, 4) float32: xyz velocity, w pressure."""
        vel = np.empty((self.particle_count(), 4), np.float32)
        self._check(self._lib.sph_download(self._ctx, None, _ptr(vel)), "sph_download")
        return vel

    def state(self):
        n = self.particle_count()
        pos = np.empty((n, 4), np.float32)
        vel = np.empty((n, 4), np.float32)
        self._check(self._lib.sph_download(self._ctx, _ptr(pos), _ptr(vel)), "sph_download")
        return pos, vel

    def previous_particles(self) -> np.ndarray:
        pos = np.empty((self.particle_count(), 4), np.float32)
        self._check(self._lib.sph_download_previous(self._ctx, _ptr(pos)), "sph_download_previous")
        return pos

    def write_instances(self, instances_ptr: int, instance_base: int = 0, sphere_mesh: int = 0,
                        tlas_ptr: int | None = None, tlas_base: int = 0, blas: int = 0, fluid_index: int = 0,
                        flags: int = 0) -> None:
        """Draw instances into device buffers (fluid_instances.comp), then keep_rendered."""
        self._check(self._lib.sph_write_instances(self._ctx, ctypes.c_void_p(instances_ptr), instance_base, sphere_mesh,
                                                  None if tlas_ptr is None else ctypes.c_void_p(tlas_ptr), tlas_base,
                                                  blas, fluid_index, flags), "sph_write_instances")

    def keep_rendered(self) -> None:
        self._check(self._lib.sph_keep_rendered(self._ctx), "sph_keep_rendered")

    def upload(self, positions: np.ndarray, velocities: np.ndarray | None = None) -> None:
        pos = np.ascontiguousarray(positions, dtype=np.float32)
        vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float32)
        if pos.ndim != 2 or pos.shape[1] != 4 or (vel is not None and vel.shape != pos.shape):
            raise ValueError("positions/velocities must be (N, 4) float32")
        self._check(self._lib.sph_upload(self._ctx, _ptr(pos), _ptr(vel), pos.shape[0]), "sph_upload")

    def upload_from(self, positions_ptr: int, velocities_ptr: int | None, count: int) -> None:
        """sph_upload from raw host addresses (e.g. pinned buffers)."""
        self._check(self._lib.sph_upload(self._ctx, ctypes.c_void_p(positions_ptr),
                                         None if velocities_ptr is None else ctypes.c_void_p(velocities_ptr), count),
                    "sph_upload")

    def download_to(self, positions_ptr: int | None, velocities_ptr: int | None) -> None:
        """sph_download into raw host addresses."""
        self._check(self._lib.sph_download(self._ctx,
                                           None if positions_ptr is None else ctypes.c_void_p(positions_ptr),
                                           None if velocities_ptr is None else ctypes.c_void_p(velocities_ptr)),
                    "sph_download")

    def step_host(self, positions_ptr: int, velocities_ptr: int | None, count: int, dt: float, substeps: int,
                  positions_out_ptr: int | None, velocities_out_ptr: int | None) -> None:
        """sph_step_host: upload from, step, and download into raw host
        addresses in one call (the copies overlap where the passes allow)."""
        def opt(p):
            return None if p is None else ctypes.c_void_p(p)

        self._check(self._lib.sph_step_host(self._ctx, ctypes.c_void_p(positions_ptr), opt(velocities_ptr), count,
                                            ctypes.c_float(dt), substeps, opt(positions_out_ptr),
                                            opt(velocities_out_ptr)), "sph_step_host")

    def step_host_arrays(self, positions: np.ndarray, velocities: np.ndarray | None, dt: float, substeps: int = 1):
        """sph_step_host on numpy (N, 4) float32 arrays; returns new arrays."""
        pos = np.ascontiguousarray(positions, dtype=np.float32)
        vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float32)
        if pos.ndim != 2 or pos.shape[1] != 4 or (vel is not None and vel.shape != pos.shape):
            raise ValueError("positions/velocities must be (N, 4) float32")
        out_p = np.empty_like(pos)
        out_v = np.empty_like(pos)
        self.step_host(pos.ctypes.data, None if vel is None else vel.ctypes.data, pos.shape[0], dt, substeps,
                       out_p.ctypes.data, out_v.ctypes.data)
        return out_p, out_v

    def synchronize(self) -> None:
        self._check(self._lib.sph_synchronize(self._ctx), "sph_synchronize")

    # -- grid and statistics ----------------------------------------------
    def grid(self):
        """FluidGrid of the last substep: (cell_of[N], cell_counts[C], cell_particles[C*32])."""
        n = self.particle_count()
        cells = self._params.lattice[3]
        cell_of = np.zeros(n, np.uint32)
        counts = np.zeros(cells, np.uint32)
        slots = np.full(cells * abi.SPH_CELL_CAPACITY, 0xFFFFFFFF, np.uint32)
        self._check(self._lib.sph_grid_download(self._ctx, _ptr(cell_of), _ptr(counts), _ptr(slots)),
                    "sph_grid_download")
        return cell_of, counts, slots

    def build_grid(self) -> None:
        self._check(self._lib.sph_grid_build(self._ctx), "sph_grid_build")

    # -- fluid surface (physics::buildFluidField / marchFluidField) ----------------
    def surface_field(self, resolution: int) -> None:
        """Samples the field of the current particles on the device."""
        self._surface_resolution = resolution
        self._check(self._lib.sph_surface_field(self._ctx, resolution), "sph_surface_field")

    def field(self) -> np.ndarray:
        """The last field, (resolution+1)^3 floats, x fastest."""
        r = getattr(self, "_surface_resolution", 0)
        out = np.empty((r + 1) ** 3, np.float32)
        self._check(self._lib.sph_surface_field_download(self._ctx, out.ctypes.data), "sph_surface_field_download")
        return out

    def surface_march(self, iso: float, capacity: int) -> int:
        """Cuts the last field on the device; returns the vertex count."""
        written = ctypes.c_uint32()
        self._check(self._lib.sph_surface_march(self._ctx, ctypes.c_float(iso), capacity, ctypes.byref(written)),
                    "sph_surface_march")
        return int(written.value)

    def surface_vertices(self, count: int) -> np.ndarray:
        out = np.zeros(count, abi.SURFACE_VERTEX)
        self._check(self._lib.sph_surface_vertices_download(self._ctx, out.ctypes.data if count else None, count),
                    "sph_surface_vertices_download")
        return out

    def surface(self, resolution: int, iso: float = 0.5, capacity: int = 196608) -> np.ndarray:
        """Field and marching cubes in one call, as the reference's CPU
        surface path does per frame (src/gfx/fluid.cpp:787-801)."""
        self.surface_field(resolution)
        return self.surface_vertices(self.surface_march(iso, capacity))

    def stats(self) -> SphStats:
        out = SphStats()
        self._check(self._lib.sph_stats_compute(self._ctx, ctypes.byref(out)), "sph_stats_compute")
        return out

    # -- device-resident access ----------------------------------------------
    def stream(self) -> int:
        out = ctypes.c_void_p()
        self._check(self._lib.sph_stream(self._ctx, ctypes.byref(out)), "sph_stream")
        return int(out.value or 0)

    def device_state(self):
        pos = ctypes.c_void_p()
        vel = ctypes.c_void_p()
        self._check(self._lib.sph_device_state(self._ctx, ctypes.byref(pos), ctypes.byref(vel)), "sph_device_state")
        return int(pos.value or 0), int(vel.value or 0)

    def tuning(self) -> dict:
        out = abi.SphTuning()
        self._check(self._lib.sph_get_tuning(self._ctx, ctypes.byref(out)), "sph_get_tuning")
        return out.as_dict()

    def set_tuning(self, **knobs) -> None:
        """Changes the launch shape (radix_bits, neighbour_kernel, block_size, queue_depth,
        schedule, sort)."""
        current = self.tuning()
        current.update(knobs)
        t = abi.SphTuning(**current)
        self._check(self._lib.sph_set_tuning(self._ctx, ctypes.byref(t)), "sph_set_tuning")

    PROFILE_PHASES = ("keys", "sort", "bounds_gather", "density", "integrate", "shapes")

    def profile(self, dt: float, substeps: int) -> dict:
        """Runs substeps phase by phase; returns total device ms per phase."""
        out = (ctypes.c_double * len(self.PROFILE_PHASES))()
        self._check(self._lib.sph_profile_substeps(self._ctx, ctypes.c_float(dt), substeps, out),
                    "sph_profile_substeps")
        return dict(zip(self.PROFILE_PHASES, list(out)))

    def launches_per_substep(self) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sph_launches_per_substep(self._ctx, ctypes.byref(out)), "sph_launches_per_substep")
        return int(out.value)

    def kernels_launched(self) -> int:
        """sph_kernels_launched: kernels enqueued so far by run (the substep
        graph) and by the processing-order remakes."""
        out = ctypes.c_uint64()
        self._check(self._lib.sph_kernels_launched(self._ctx, ctypes.byref(out)), "sph_kernels_launched")
        return out.value

    def device_bytes(self) -> int:
        out = ctypes.c_uint64()
        self._check(self._lib.sph_device_bytes(self._ctx, ctypes.byref(out)), "sph_device_bytes")
        return int(out.value)
