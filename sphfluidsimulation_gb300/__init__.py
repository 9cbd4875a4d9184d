"""GB300-native SPH step engine.

A drop-in third engine for the SPH::SimulationEngine interface of
Murk42/SPHFluidSimulation: hand-written sm_103a CUDA kernels behind the C ABI
in include/sph_gb300.h (libsph_gb300.so), with this package as a thin Python
binding, the synthetic scene generators, and the serving loop driver.
"""
from . import scenes  # noqa: F401

__all__ = ["scenes", "engine", "build"]
