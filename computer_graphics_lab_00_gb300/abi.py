"""ctypes mirror of include/sph_c.h and the loader of the native library.

The structures here are byte-for-byte the C structs of `sph_c.h`, which in
turn carry the scalar layout of the reference's `gfx::GpuFluidParams`
(src/gfx/fluid.h:81-102). Nothing in this module touches torch: the boundary
is plain pointers and sizes.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PACKAGE_DIR = Path(__file__).resolve().parent
NATIVE_DIR = PACKAGE_DIR / "_native"
LIBRARY_NAME = "libsph_gb300.so"

SPH_ABI_VERSION = 1
SPH_CELL_CAPACITY = 32
SPH_MAX_COLLIDERS = 8
SPH_MAX_FORCE_FIELDS = 8
SPH_STATIC_MAX_PARTICLES = 65536
SPH_STATIC_MAX_CELLS = 65536

SPH_OK = 0
SPH_ERR_INVALID_ARGUMENT = -1
SPH_ERR_CAPACITY = -2
SPH_ERR_CUDA = -3
SPH_ERR_OUT_OF_MEMORY = -4
SPH_ERR_UNSUPPORTED = -5
SPH_ERR_TIMEOUT = -6
SPH_ERR_NO_DEVICE = -7
SPH_ERR_NONFINITE = -8
SPH_ALL_TANKS = 0xFFFFFFFF


class SphCollider(ctypes.Structure):
    _fields_ = [
        ("data0", ctypes.c_float * 4),
        ("inverse_world", ctypes.c_float * 16),
        ("world", ctypes.c_float * 16),
        ("type", ctypes.c_uint32),
        ("pad", ctypes.c_uint32 * 3),
    ]


class SphForceField(ctypes.Structure):
    _fields_ = [
        ("position_radius", ctypes.c_float * 4),
        ("axis_strength", ctypes.c_float * 4),
        ("falloff", ctypes.c_float),
        ("type", ctypes.c_uint32),
        ("pad", ctypes.c_uint32 * 2),
    ]


class SphParams(ctypes.Structure):
    _fields_ = [
        ("emitter_world", ctypes.c_float * 16),
        ("emitter_half_extents", ctypes.c_float * 4),
        ("container_min", ctypes.c_float * 4),
        ("container_max", ctypes.c_float * 4),
        ("gravity", ctypes.c_float * 4),
        ("smoothing_radius", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("stiffness", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("lattice", ctypes.c_uint32 * 4),
        ("collider_count", ctypes.c_uint32),
        ("pad0", ctypes.c_uint32),
        ("pad1", ctypes.c_uint32),
        ("pad2", ctypes.c_uint32),
        ("colliders", SphCollider * SPH_MAX_COLLIDERS),
        ("field_count", ctypes.c_uint32),
        ("field_pad0", ctypes.c_uint32),
        ("field_pad1", ctypes.c_uint32),
        ("field_pad2", ctypes.c_uint32),
        ("fields", SphForceField * SPH_MAX_FORCE_FIELDS),
    ]

    # Convenience accessors named after physics::FluidParams (fluid_sph.h:42-67).
    @property
    def spacing(self) -> float:
        return self.emitter_half_extents[3]

    @property
    def particle_radius(self) -> float:
        return self.container_min[3]

    @property
    def wall_restitution(self) -> float:
        return self.container_max[3]

    @property
    def particle_mass(self) -> float:
        return self.gravity[3]

    @property
    def cell_count(self) -> int:
        return self.lattice[3]

    def copy(self) -> "SphParams":
        out = SphParams()
        ctypes.memmove(ctypes.byref(out), ctypes.byref(self), ctypes.sizeof(SphParams))
        return out


class SphFluidSettings(ctypes.Structure):
    _fields_ = [
        ("emitter_half_extents", ctypes.c_float * 3),
        ("particle_radius", ctypes.c_float),
        ("smoothing_radius", ctypes.c_float),
        ("rest_density", ctypes.c_float),
        ("stiffness", ctypes.c_float),
        ("viscosity", ctypes.c_float),
        ("container_min", ctypes.c_float * 3),
        ("container_max", ctypes.c_float * 3),
        ("gravity", ctypes.c_float * 3),
    ]


class SphTuning(ctypes.Structure):
    _fields_ = [
        ("radix_bits", ctypes.c_uint32),
        ("neighbour_kernel", ctypes.c_uint32),
        ("block_size", ctypes.c_uint32),
        ("queue_depth", ctypes.c_uint32),
        ("schedule", ctypes.c_uint32),
        ("sort", ctypes.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class SphStats(ctypes.Structure):
    _fields_ = [
        ("particles", ctypes.c_uint32),
        ("buckets", ctypes.c_uint32),
        ("max_bucket_count", ctypes.c_uint32),
        ("overflow_buckets", ctypes.c_uint32),
        ("candidates", ctypes.c_uint64),
        ("pairs_in_range", ctypes.c_uint64),
        ("mean_density", ctypes.c_double),
        ("mean_compression", ctypes.c_double),
        ("max_density", ctypes.c_double),
        ("centre_of_mass", ctypes.c_double * 3),
        ("kinetic_energy", ctypes.c_double),
        ("nonfinite", ctypes.c_uint32),
        ("pad", ctypes.c_uint32),
    ]


# SphStats as a numpy record: a batch's statistics read as one array.
STATS_DTYPE = np.dtype([("particles", "<u4"), ("buckets", "<u4"), ("max_bucket_count", "<u4"),
                        ("overflow_buckets", "<u4"), ("candidates", "<u8"), ("pairs_in_range", "<u8"),
                        ("mean_density", "<f8"), ("mean_compression", "<f8"), ("max_density", "<f8"),
                        ("centre_of_mass", "<f8", (3,)), ("kinetic_energy", "<f8"), ("nonfinite", "<u4"),
                        ("pad", "<u4")])
assert STATS_DTYPE.itemsize == ctypes.sizeof(SphStats)

assert ctypes.sizeof(SphCollider) == 160
assert ctypes.sizeof(SphForceField) == 48
assert ctypes.sizeof(SphParams) == 1856


# physics::SurfaceVertex / sph_surface_vertex: xyz position, packed unit normal.
SURFACE_VERTEX = np.dtype([("position", np.float32, 3), ("normal", np.uint32)])
assert SURFACE_VERTEX.itemsize == 16
SPH_MC_TABLE_WIDTH = 16
SPH_SURFACE_MAX_RESOLUTION = 640


# gfx::GpuInstance and the TLAS record (sph_instance / sph_tlas_instance).
INSTANCE = np.dtype([("model", np.float32, 16), ("previous_model", np.float32, 16), ("normal_matrix", np.float32, 16),
                     ("mesh_index", np.uint32), ("bucket", np.uint32), ("bucket_base", np.uint32),
                     ("joint_offset", np.uint32), ("skinned_vertex_offset", np.uint32),
                     ("previous_skinned_vertex_offset", np.uint32), ("skinned_meshlet_offset", np.uint32),
                     ("visibility_base", np.uint32)])
TLAS_INSTANCE = np.dtype([("transform", np.float32, 12), ("custom_index_mask", np.uint32),
                          ("sbt_offset_flags", np.uint32), ("blas", np.uint64)])
assert INSTANCE.itemsize == 224 and TLAS_INSTANCE.itemsize == 64
SPH_INSTANCES_RESET_HISTORY = 1
SPH_INSTANCES_WRITE_TLAS = 2
SPH_INSTANCES_SURFACE_TLAS = 4


class SphError(RuntimeError):
    """A non-zero status from the native library."""

    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        text = f"{what}: status {status}"
        if detail:
            text += f" ({detail})"
        super().__init__(text)


_lib = None


def library_path() -> Path:
    override = os.environ.get("SPH_GB300_LIBRARY")
    return Path(override) if override else NATIVE_DIR / LIBRARY_NAME


def load() -> ctypes.CDLL:
    """Loads the CUDA library; raises if it was not built (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not path.exists():
        raise RuntimeError(
            f"native SPH library missing at {path}; build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or "
            "`python -m computer_graphics_lab_00_gb300.build`"
        )
    lib = ctypes.CDLL(str(path))
    _declare(lib)
    if lib.sph_abi_version() != SPH_ABI_VERSION:
        raise RuntimeError(f"{path}: ABI {lib.sph_abi_version()} != {SPH_ABI_VERSION}")
    _lib = lib
    return lib


def _declare(lib: ctypes.CDLL) -> None:
    P = ctypes.POINTER
    c_int, c_u32, c_f32, c_void_p = ctypes.c_int, ctypes.c_uint32, ctypes.c_float, ctypes.c_void_p
    f32p = P(ctypes.c_float)
    u32p = P(ctypes.c_uint32)
    sigs = {
        "sph_abi_version": (c_int, []),
        "sph_status_string": (ctypes.c_char_p, [c_int]),
        "sph_last_error": (ctypes.c_char_p, [c_void_p]),
        "sph_derive_params": (c_int, [P(SphFluidSettings), f32p, c_u32, c_u32, P(SphParams)]),
        "sph_fluid_substeps": (c_int, [P(SphParams), c_f32, u32p]),
        "sph_cell_count_for": (c_u32, [c_u32]),
        "sph_cell_count_uncapped": (c_u32, [c_u32]),
        "sph_create": (c_int, [P(SphParams), c_u32, c_int, P(c_void_p)]),
        "sph_destroy": (c_int, [c_void_p]),
        "sph_set_params": (c_int, [c_void_p, P(SphParams)]),
        "sph_particle_count": (c_int, [c_void_p, u32p]),
        "sph_emit": (c_int, [c_void_p, c_u32]),
        "sph_upload": (c_int, [c_void_p, c_void_p, c_void_p, c_u32]),
        "sph_download": (c_int, [c_void_p, c_void_p, c_void_p]),
        "sph_step_host": (c_int, [c_void_p, c_void_p, c_void_p, c_u32, c_f32, c_u32, c_void_p, c_void_p]),
        "sph_step": (c_int, [c_void_p, c_f32]),
        "sph_substep": (c_int, [c_void_p, c_f32]),
        "sph_keep_rendered": (c_int, [c_void_p]),
        "sph_download_previous": (c_int, [c_void_p, c_void_p]),
        "sph_synchronize": (c_int, [c_void_p]),
        "sph_grid_download": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
        "sph_grid_build": (c_int, [c_void_p]),
        "sph_grid_build_static": (c_int, [P(SphParams), c_void_p, c_u32, c_void_p, c_void_p, c_void_p, c_void_p]),
        "sph_stats_compute": (c_int, [c_void_p, P(SphStats)]),
        "sph_write_instances": (c_int, [c_void_p, c_void_p, c_u32, c_u32, c_void_p, c_u32, ctypes.c_uint64, c_u32,
                                        c_u32]),
        "sph_surface_table": (c_int, [c_void_p]),
        "sph_surface_field": (c_int, [c_void_p, c_u32]),
        "sph_surface_field_download": (c_int, [c_void_p, c_void_p]),
        "sph_surface_march": (c_int, [c_void_p, ctypes.c_float, c_u32, P(c_u32)]),
        "sph_surface_vertices_download": (c_int, [c_void_p, c_void_p, c_u32]),
        "sph_surface_device": (c_int, [c_void_p, P(c_void_p), P(c_void_p)]),
        "sph_march_field": (c_int, [c_void_p, c_u32, c_void_p, c_void_p, ctypes.c_float, c_void_p, c_u32, P(c_u32),
                                    c_int]),
        "sph_stream": (c_int, [c_void_p, P(c_void_p)]),
        "sph_device_state": (c_int, [c_void_p, P(c_void_p), P(c_void_p)]),
        "sph_run": (c_int, [c_void_p, c_f32, c_u32]),
        "sph_profile_substeps": (c_int, [c_void_p, c_f32, c_u32, P(ctypes.c_double)]),
        "sph_get_tuning": (c_int, [c_void_p, P(SphTuning)]),
        "sph_set_tuning": (c_int, [c_void_p, P(SphTuning)]),
        "sph_selftest_division": (c_int, [c_void_p, ctypes.c_uint64, ctypes.c_uint64, c_int, P(ctypes.c_uint64)]),
        "sph_launches_per_substep": (c_int, [c_void_p, u32p]),
        "sph_kernels_launched": (c_int, [c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
        "sph_device_bytes": (c_int, [c_void_p, P(ctypes.c_uint64)]),
    }
    u8p = P(ctypes.c_uint8)
    f64p = P(ctypes.c_double)
    tp = P(SphTuning)
    sigs.update({
        "sph_autotune": (c_int, [c_void_p, c_f32, c_u32, tp, f32p]),
        "sph_batch_create": (c_int, [P(SphParams), u32p, c_u32, c_int, P(c_void_p)]),
        "sph_batch_destroy": (c_int, [c_void_p]),
        "sph_batch_last_error": (ctypes.c_char_p, [c_void_p]),
        "sph_batch_tank_count": (c_int, [c_void_p, u32p]),
        "sph_batch_particle_count": (c_int, [c_void_p, c_u32, u32p]),
        "sph_batch_upload": (c_int, [c_void_p, c_u32, c_void_p, c_void_p]),
        "sph_batch_download": (c_int, [c_void_p, c_u32, c_void_p, c_void_p]),
        "sph_batch_emit": (c_int, [c_void_p, c_u32]),
        "sph_batch_set_active": (c_int, [c_void_p, u8p]),
        "sph_batch_run": (c_int, [c_void_p, c_f32, c_u32]),
        "sph_batch_run_per_tank": (c_int, [c_void_p, f32p, u32p]),
        "sph_batch_step": (c_int, [c_void_p, c_f32]),
        "sph_batch_stats": (c_int, [c_void_p, P(SphStats)]),
        "sph_batch_synchronize": (c_int, [c_void_p]),
        "sph_batch_stream": (c_int, [c_void_p, P(c_void_p)]),
        "sph_batch_get_tuning": (c_int, [c_void_p, tp]),
        "sph_batch_set_tuning": (c_int, [c_void_p, tp]),
        "sph_batch_autotune": (c_int, [c_void_p, c_f32, c_u32, tp, f32p]),
        "sph_batch_profile_substeps": (c_int, [c_void_p, c_f32, c_u32, f64p]),
        "sph_batch_launches_per_substep": (c_int, [c_void_p, u32p]),
        "sph_batch_device_bytes": (c_int, [c_void_p, P(ctypes.c_uint64)]),
        "sph_run_learned": (c_int, [c_void_p, c_f32, c_u32, c_void_p]),
        "sph_batch_run_learned": (c_int, [c_void_p, c_f32, c_u32, c_void_p]),
        "sph_batch_learned_features": (c_int, [c_void_p, c_f32, c_void_p]),
        "sph_batch_learned_correction": (c_int, [c_void_p, c_f32, c_void_p, c_void_p]),
        "sph_batch_learned_check": (c_int, [c_void_p]),
        "sph_batch_snapshot": (c_int, [c_void_p, c_u32, c_int]),
        "sph_batch_restore_tanks": (c_int, [c_void_p, c_u32, u8p]),
        "sph_batch_device_state": (c_int, [c_void_p, P(c_void_p), P(c_void_p)]),
        "sph_batch_tank_offset": (c_int, [c_void_p, c_u32, u32p]),
        "sph_batch_copy_state": (c_int, [c_void_p, c_void_p, c_void_p]),
    })
    for name, (restype, argtypes) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes


def check(status: int, what: str, ctx=None) -> None:
    if status != SPH_OK:
        lib = load()
        detail = lib.sph_status_string(status).decode()
        if ctx is not None:
            last = lib.sph_last_error(ctx).decode()
            if last:
                detail += "; " + last
        raise SphError(status, what, detail)
