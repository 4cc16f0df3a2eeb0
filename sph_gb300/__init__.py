"""sph_gb300 -- GB300-native SPH compute step (TinySPH's hash.c + fluid.c step).

The product is libsph_cuda (sph_gb300/lib/libsph_cuda.so, C ABI in
include/sph_cuda.h, include/sph_legacy.h and include/sph_learned.h).  This package builds it and
wraps it for Python callers; it contains no CPU implementation of the step.
"""
from . import scenes
from ._lib import PARTICLE_DTYPE, SphError, lib
from .simulation import Ensemble, LearnedModel, Simulation, gemm_check, render_liquid, write_ppm

__all__ = ["Simulation", "Ensemble", "LearnedModel", "gemm_check", "render_liquid", "write_ppm", "SphError", "PARTICLE_DTYPE", "scenes", "lib"]
