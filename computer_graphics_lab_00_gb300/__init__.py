"""GB300-native SPH fluid step (drop-in for the reference's physics::FluidSolver).

The compute path is libsph_gb300.so: hand-written CUDA kernels for sm_103a
behind the C ABI of include/sph_c.h. This package holds the ctypes mirror of
that ABI (`abi`), the Python twin of the reference's FluidSolver API
(`fluid`), the seeded synthetic workloads (`workloads`) and the build
script (`build`).
"""
from .abi import SphError, SphFluidSettings, SphParams, SphStats  # noqa: F401

__all__ = ["SphError", "SphFluidSettings", "SphParams", "SphStats"]
