"""The learned acceleration correction over the C ABI (sph_mlp_*).

`MlpGpu` owns one 32 -> 128 -> 128 -> 3 MLP on a GPU: tensor-core forward,
FP32 backward and Adam, parameters as one FP32 vector (SPH_MLP_PARAMS) that
can be saved and loaded. Feature and target arrays passed to it are device
pointers (for example torch CUDA tensors' data_ptr()).
"""
from __future__ import annotations

import ctypes
import json
from pathlib import Path

import numpy as np

from . import abi
from .abi import load

INPUTS = 32
HIDDEN = 128
OUTPUTS = 3
PARAMS = 32 * 128 + 128 + 128 * 128 + 128 + 3 * 128 + 3

_declared = False


def _declare(lib):
    global _declared
    if _declared:
        return
    P = ctypes.POINTER
    f32p = P(ctypes.c_float)
    sigs = {
        "sph_mlp_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, P(ctypes.c_void_p)]),
        "sph_mlp_destroy": (ctypes.c_int, [ctypes.c_void_p]),
        "sph_mlp_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
        "sph_mlp_get_params": (ctypes.c_int, [ctypes.c_void_p, f32p]),
        "sph_mlp_set_params": (ctypes.c_int, [ctypes.c_void_p, f32p]),
        "sph_mlp_set_normalisation": (ctypes.c_int, [ctypes.c_void_p, f32p, f32p, f32p]),
        "sph_mlp_get_normalisation": (ctypes.c_int, [ctypes.c_void_p, f32p, f32p, f32p]),
        "sph_mlp_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                           ctypes.c_void_p]),
        "sph_mlp_gradients": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, f32p,
                                             f32p]),
        "sph_mlp_set_adam": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
        "sph_mlp_train_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                              ctypes.c_float, f32p]),
        "sph_mlp_stream": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_void_p)]),
        "sph_mlp_selftest_erf": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, f32p]),
        "sph_mlp_apply_gradients": (ctypes.c_int, [ctypes.c_void_p, f32p, ctypes.c_float]),
        "sph_mlp_set_net_force_free": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32]),
        "sph_mlp_selftest_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int]),
    }
    for name, (restype, argtypes) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    _declared = True


def _fp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class MlpGpu:
    """One MLP on one GPU."""

    def __init__(self, device: int = 0, seed: int = 0):
        self._lib = load()
        _declare(self._lib)
        self._h = ctypes.c_void_p()
        self.free_axes = 0
        self._check(self._lib.sph_mlp_create(device, seed, ctypes.byref(self._h)), "sph_mlp_create")

    def close(self):
        if self._h:
            self._lib.sph_mlp_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def _check(self, status: int, what: str):
        if status != abi.SPH_OK:
            detail = self._lib.sph_status_string(status).decode()
            if self._h:
                last = self._lib.sph_mlp_last_error(self._h).decode()
                detail += f"; {last}" if last else ""
            raise abi.SphError(status, what, detail)

    def params(self) -> np.ndarray:
        out = np.empty(PARAMS, np.float32)
        self._check(self._lib.sph_mlp_get_params(self._h, _fp(out)), "sph_mlp_get_params")
        return out

    def set_params(self, params) -> None:
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.shape != (PARAMS,):
            raise ValueError(f"expected {PARAMS} parameters")
        self._check(self._lib.sph_mlp_set_params(self._h, _fp(p)), "sph_mlp_set_params")

    def set_normalisation(self, mean, std, scale) -> None:
        m = np.ascontiguousarray(mean, np.float32)
        s = np.ascontiguousarray(std, np.float32)
        o = np.ascontiguousarray(scale, np.float32)
        self._check(self._lib.sph_mlp_set_normalisation(self._h, _fp(m), _fp(s), _fp(o)), "sph_mlp_set_normalisation")

    def normalisation(self):
        m = np.empty(INPUTS, np.float32)
        s = np.empty(INPUTS, np.float32)
        o = np.empty(OUTPUTS, np.float32)
        self._check(self._lib.sph_mlp_get_normalisation(self._h, _fp(m), _fp(s), _fp(o)), "sph_mlp_get_normalisation")
        return m, s, o

    def forward(self, features_ptr: int, count: int, out_ptr: int, stream: int | None = None) -> None:
        self._check(self._lib.sph_mlp_forward(self._h, ctypes.c_void_p(features_ptr), count, ctypes.c_void_p(out_ptr),
                                              None if stream is None else ctypes.c_void_p(stream)), "sph_mlp_forward")

    def gradients(self, features_ptr: int, targets_ptr: int, count: int):
        g = np.empty(PARAMS, np.float32)
        loss = np.empty(1, np.float32)
        self._check(self._lib.sph_mlp_gradients(self._h, ctypes.c_void_p(features_ptr), ctypes.c_void_p(targets_ptr),
                                                count, _fp(g), _fp(loss)), "sph_mlp_gradients")
        return float(loss[0]), g

    def set_adam(self, beta1: float = 0.9, beta2: float = 0.999, epsilon: float = 1e-8) -> None:
        self._check(self._lib.sph_mlp_set_adam(self._h, beta1, beta2, epsilon), "sph_mlp_set_adam")

    def train_step(self, features_ptr: int, targets_ptr: int, count: int, lr: float = 1e-3) -> float:
        loss = np.empty(1, np.float32)
        self._check(self._lib.sph_mlp_train_step(self._h, ctypes.c_void_p(features_ptr), ctypes.c_void_p(targets_ptr),
                                                 count, lr, _fp(loss)), "sph_mlp_train_step")
        return float(loss[0])

    def set_net_force_free(self, axes: int) -> None:
        """Learned steps take each tank's mean correction off along the axes
        in the mask (bit 0 x, 1 y, 2 z; 0 keeps it)."""
        self._check(self._lib.sph_mlp_set_net_force_free(self._h, axes), "sph_mlp_set_net_force_free")
        self.free_axes = int(axes)

    def apply_gradients(self, grads, lr: float = 1e-3) -> None:
        """Adam with an externally reduced gradient (data-parallel training)."""
        g = np.ascontiguousarray(grads, dtype=np.float32)
        if g.shape != (PARAMS,):
            raise ValueError(f"expected {PARAMS} gradient entries")
        self._check(self._lib.sph_mlp_apply_gradients(self._h, _fp(g), lr), "sph_mlp_apply_gradients")

    def selftest_erf(self, count: int = 1 << 24) -> float:
        out = np.zeros(1, np.float32)
        self._check(self._lib.sph_mlp_selftest_erf(self._h, count, _fp(out)), "sph_mlp_selftest_erf")
        return float(out[0])

    def selftest_wait(self, polls: int, arrive: bool) -> int:
        """Status of a bounded mbarrier wait (SPH_OK or SPH_ERR_TIMEOUT)."""
        return int(self._lib.sph_mlp_selftest_wait(self._h, polls, 1 if arrive else 0))

    # -- checkpoints: FP32 weights + normalisation, JSON ----------------------------
    def save(self, path) -> None:
        m, s, o = self.normalisation()
        Path(path).write_text(json.dumps({"params": self.params().tolist(), "feature_mean": m.tolist(),
                                          "feature_std": s.tolist(), "output_scale": o.tolist()}))

    def load(self, path) -> None:
        data = json.loads(Path(path).read_text())
        self.set_params(np.array(data["params"], np.float32))
        self.set_normalisation(data["feature_mean"], data["feature_std"], data["output_scale"])
