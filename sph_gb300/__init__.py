"""sph_gb300 -- GB300-native SPH compute step (TinySPH's hash.c + fluid.c step).

The product is libsph_cuda (sph_gb300/lib/libsph_cuda.so, C ABI in
include/sph_cuda.h and include/sph_legacy.h).  This package builds it and
wraps it for Python callers; it contains no CPU implementation of the step.
"""
from . import scenes
from ._lib import PARTICLE_DTYPE, SphError, lib
from .simulation import Ensemble, Simulation

__all__ = ["Simulation", "Ensemble", "SphError", "PARTICLE_DTYPE", "scenes", "lib"]
