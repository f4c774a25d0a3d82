"""Batched tanks over the C ABI: many independent fluids advanced by one CUDA
graph launch per substep (sph_batch_* in include/sph_c.h).

Each tank keeps the semantics of one `physics::FluidSolver`
(src/physics/fluid_sph.cpp:190-321) bit for bit; the batch only shares the
launches. Autotuning results can be cached per workload in a JSON file.
"""
from __future__ import annotations

import ctypes
import json
import os
from pathlib import Path

import numpy as np

from . import abi
from .abi import SphParams, SphStats, SphTuning, check, load


def _ptr(a: np.ndarray | None):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


class BatchSolverGpu:
    """A set of tanks on one GPU."""

    PROFILE_PHASES = ("keys", "sort", "bounds_gather", "density", "integrate", "shapes")

    def __init__(self, params: list[SphParams], counts: list[int], device: int = 0):
        if len(params) != len(counts) or not params:
            raise ValueError("one SphParams per tank and at least one tank")
        self._lib = load()
        self._handle = ctypes.c_void_p()
        arr = (SphParams * len(params))(*[p.copy() for p in params])
        cnt = (ctypes.c_uint32 * len(counts))(*[int(c) for c in counts])
        check(self._lib.sph_batch_create(arr, cnt, len(params), device, ctypes.byref(self._handle)),
              "sph_batch_create")
        self.params = [p.copy() for p in params]
        self.counts = [int(c) for c in counts]

    def close(self) -> None:
        if self._handle:
            self._lib.sph_batch_destroy(self._handle)
            self._handle = ctypes.c_void_p()

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
        if status != abi.SPH_OK:
            detail = self._lib.sph_status_string(status).decode()
            last = self._lib.sph_batch_last_error(self._handle).decode()
            raise abi.SphError(status, what, detail + (f"; {last}" if last else ""))

    @property
    def tanks(self) -> int:
        return len(self.counts)

    @property
    def total_particles(self) -> int:
        return sum(self.counts)

    def upload(self, tank: int, positions: np.ndarray, velocities: np.ndarray | None = None) -> None:
        pos = np.ascontiguousarray(positions, dtype=np.float32)
        vel = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float32)
        if pos.shape != (self.counts[tank], 4):
            raise ValueError(f"tank {tank} holds {self.counts[tank]} particles")
        self._check(self._lib.sph_batch_upload(self._handle, tank, _ptr(pos), _ptr(vel)), "sph_batch_upload")

    def download(self, tank: int):
        pos = np.empty((self.counts[tank], 4), np.float32)
        vel = np.empty((self.counts[tank], 4), np.float32)
        self._check(self._lib.sph_batch_download(self._handle, tank, _ptr(pos), _ptr(vel)), "sph_batch_download")
        return pos, vel

    def emit(self, tank: int) -> None:
        self._check(self._lib.sph_batch_emit(self._handle, tank), "sph_batch_emit")

    def set_active(self, active) -> None:
        a = np.ascontiguousarray(np.asarray(active, dtype=np.uint8))
        if a.shape != (self.tanks,):
            raise ValueError("one flag per tank")
        self._check(self._lib.sph_batch_set_active(self._handle, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
                    "sph_batch_set_active")

    def run(self, dt: float, substeps: int) -> None:
        self._check(self._lib.sph_batch_run(self._handle, ctypes.c_float(dt), substeps), "sph_batch_run")

    def run_per_tank(self, dt, substeps) -> None:
        d = np.ascontiguousarray(np.asarray(dt, dtype=np.float32))
        n = np.ascontiguousarray(np.asarray(substeps, dtype=np.uint32))
        self._check(self._lib.sph_batch_run_per_tank(self._handle, d.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                     n.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))),
                    "sph_batch_run_per_tank")

    def step(self, delta_seconds: float) -> None:
        self._check(self._lib.sph_batch_step(self._handle, ctypes.c_float(delta_seconds)), "sph_batch_step")

    def stats(self) -> list[SphStats]:
        out = (SphStats * self.tanks)()
        self._check(self._lib.sph_batch_stats(self._handle, out), "sph_batch_stats")
        return list(out)

    def stats_array(self) -> np.ndarray:
        """The same statistics as one numpy record array (abi.STATS_DTYPE),
        without a Python object per tank."""
        out = np.zeros(self.tanks, abi.STATS_DTYPE)
        self._check(self._lib.sph_batch_stats(self._handle, out.ctypes.data_as(ctypes.POINTER(SphStats))),
                    "sph_batch_stats")
        return out

    def synchronize(self) -> None:
        self._check(self._lib.sph_batch_synchronize(self._handle), "sph_batch_synchronize")

    def stream(self) -> int:
        out = ctypes.c_void_p()
        self._check(self._lib.sph_batch_stream(self._handle, ctypes.byref(out)), "sph_batch_stream")
        return int(out.value or 0)

    def tuning(self) -> dict:
        out = SphTuning()
        self._check(self._lib.sph_batch_get_tuning(self._handle, ctypes.byref(out)), "sph_batch_get_tuning")
        return out.as_dict()

    def set_tuning(self, **knobs) -> None:
        current = self.tuning()
        current.update(knobs)
        t = SphTuning(**current)
        self._check(self._lib.sph_batch_set_tuning(self._handle, ctypes.byref(t)), "sph_batch_set_tuning")

    def autotune(self, dt: float, substeps_per_trial: int = 5, cache: str | os.PathLike | None = None,
                 key: str | None = None) -> dict:
        """Picks the fastest launch shape (state restored afterwards).

        With `cache` and `key`, a stored choice for `key` is applied without
        measuring, and a new measurement is stored under `key`.
        """
        if cache is not None and key is not None:
            path = Path(cache)
            if path.exists():
                stored = json.loads(path.read_text()).get(key)
                if stored:
                    self.set_tuning(**stored["tuning"])
                    return stored
        best = SphTuning()
        ms = ctypes.c_float()
        self._check(self._lib.sph_batch_autotune(self._handle, ctypes.c_float(dt), substeps_per_trial,
                                                 ctypes.byref(best), ctypes.byref(ms)), "sph_batch_autotune")
        result = {"tuning": best.as_dict(), "ms_per_substep": float(ms.value)}
        if cache is not None and key is not None:
            path = Path(cache)
            data = json.loads(path.read_text()) if path.exists() else {}
            data[key] = result
            path.write_text(json.dumps(data, indent=1, sort_keys=True))
        return result

    def profile(self, dt: float, substeps: int) -> dict:
        out = (ctypes.c_double * len(self.PROFILE_PHASES))()
        self._check(self._lib.sph_batch_profile_substeps(self._handle, ctypes.c_float(dt), substeps, out),
                    "sph_batch_profile_substeps")
        return dict(zip(self.PROFILE_PHASES, list(out)))

    # -- learned coarse step --------------------------------------------------------
    def run_learned(self, dt: float, substeps: int, mlp=None) -> None:
        """Learned coarse substeps (mlp None: zero correction, = plain bits)."""
        handle = None if mlp is None else mlp.handle
        self._check(self._lib.sph_batch_run_learned(self._handle, ctypes.c_float(dt), substeps, handle),
                    "sph_batch_run_learned")

    def learned_features(self, dt: float, features_ptr: int) -> None:
        self._check(self._lib.sph_batch_learned_features(self._handle, ctypes.c_float(dt),
                                                         ctypes.c_void_p(features_ptr)), "sph_batch_learned_features")

    def learned_correction(self, dt: float, mlp, correction_ptr: int) -> None:
        """The correction (float4 per particle, id order, device) a learned
        substep of length dt would add to the current state."""
        self._check(self._lib.sph_batch_learned_correction(self._handle, ctypes.c_float(dt), mlp.handle,
                                                           ctypes.c_void_p(correction_ptr)),
                    "sph_batch_learned_correction")

    def learned_check(self) -> None:
        self._check(self._lib.sph_batch_learned_check(self._handle), "sph_batch_learned_check")

    def snapshot(self, slot: int = 0, save: bool = True) -> None:
        self._check(self._lib.sph_batch_snapshot(self._handle, slot, 1 if save else 0), "sph_batch_snapshot")

    def restore_tanks(self, slot: int, which) -> None:
        w = np.ascontiguousarray(np.asarray(which, dtype=np.uint8))
        self._check(self._lib.sph_batch_restore_tanks(self._handle, slot,
                                                      w.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
                    "sph_batch_restore_tanks")

    def device_state(self):
        pos = ctypes.c_void_p()
        vel = ctypes.c_void_p()
        self._check(self._lib.sph_batch_device_state(self._handle, ctypes.byref(pos), ctypes.byref(vel)),
                    "sph_batch_device_state")
        return int(pos.value or 0), int(vel.value or 0)

    def copy_state(self, positions_ptr: int | None, velocities_ptr: int | None) -> None:
        """Device-to-device copy of all tanks' state (id order) on the batch stream."""
        self._check(self._lib.sph_batch_copy_state(self._handle,
                                                   None if positions_ptr is None else ctypes.c_void_p(positions_ptr),
                                                   None if velocities_ptr is None else ctypes.c_void_p(velocities_ptr)),
                    "sph_batch_copy_state")

    def tank_offset(self, tank: int) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sph_batch_tank_offset(self._handle, tank, ctypes.byref(out)), "sph_batch_tank_offset")
        return int(out.value)

    def launches_per_substep(self) -> int:
        out = ctypes.c_uint32()
        self._check(self._lib.sph_batch_launches_per_substep(self._handle, ctypes.byref(out)),
                    "sph_batch_launches_per_substep")
        return int(out.value)

    def device_bytes(self) -> int:
        out = ctypes.c_uint64()
        self._check(self._lib.sph_batch_device_bytes(self._handle, ctypes.byref(out)), "sph_batch_device_bytes")
        return int(out.value)
