"""ctypes binding of libsph_cuda (include/sph_cuda.h, include/sph_legacy.h).

Loading fails loudly when the in-tree library is missing: there is no CPU
implementation behind this package.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
# SPH_CUDA_LIB selects another build of the library (e.g. the bounds-checked
# lib/libsph_cuda_checked.so) for this process.
LIB_PATH = os.environ.get("SPH_CUDA_LIB") or os.path.join(PKG, "lib", "libsph_cuda.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)
c_short_p = ctypes.POINTER(ctypes.c_short)


class FluidParticle(ctypes.Structure):
    """fluid_particle, fluid.h:56-70 (52 bytes)."""
    _fields_ = [(n, ctypes.c_float) for n in (
        "x_prev", "y_prev", "x", "y", "v_x", "v_y", "a_x", "a_y", "density", "density_near",
        "pressure", "pressure_near")] + [("id", ctypes.c_int)]


PARTICLE_DTYPE = np.dtype([(n, "<f4") for n, _ in FluidParticle._fields_[:-1]] + [("id", "<i4")])
assert PARTICLE_DTYPE.itemsize == 52


class TunableParameters(ctypes.Structure):
    """tunable_parameters, fluid.h:78-97 (64 bytes)."""
    _fields_ = [(n, ctypes.c_float) for n in (
        "rest_density", "smoothing_radius", "g", "k", "k_near", "k_spring", "sigma", "beta",
        "time_step", "node_start_x", "node_end_x", "mover_center_x", "mover_center_y",
        "mover_width", "mover_height")] + [
        ("mover_type", ctypes.c_byte), ("kill_sim", ctypes.c_byte), ("active", ctypes.c_byte)]


class Param(ctypes.Structure):
    """param, fluid.h:100-106 (80 bytes)."""
    _fields_ = [("tunable_params", TunableParameters),
                ("number_fluid_particles_global", ctypes.c_int),
                ("number_fluid_particles_local", ctypes.c_int),
                ("max_fluid_particle_index", ctypes.c_int),
                ("number_halo_particles", ctypes.c_int)]


class AABB(ctypes.Structure):
    """AABB_t, geometry.h:33-40."""
    _fields_ = [(n, ctypes.c_float) for n in ("min_x", "max_x", "min_y", "max_y", "min_z", "max_z")]


class Neighbor(ctypes.Structure):
    """neighbor, fluid.h:72-75."""
    _fields_ = [("fluid_neighbors", ctypes.POINTER(ctypes.POINTER(FluidParticle))),
                ("number_fluid_neighbors", ctypes.c_int)]


class Bucket(ctypes.Structure):
    """bucket_t, hash.h:35-38."""
    _fields_ = [("fluid_particles", ctypes.POINTER(ctypes.POINTER(FluidParticle))),
                ("number_fluid", ctypes.c_uint)]


class NeighborGrid(ctypes.Structure):
    """neighbor_grid_t, hash.h:40-48."""
    _fields_ = [("spacing", ctypes.c_float), ("size_x", ctypes.c_uint), ("size_y", ctypes.c_uint),
                ("neighbors", ctypes.POINTER(Neighbor)), ("grid_buckets", ctypes.POINTER(Bucket)),
                ("max_neighbors", ctypes.c_uint), ("max_bucket_size", ctypes.c_uint)]


class SceneDesc(ctypes.Structure):
    """sph_scene_desc (include/sph_cuda.h): one scene of an ensemble."""
    _fields_ = [("params", TunableParameters), ("boundary", AABB), ("spacing", ctypes.c_float),
                ("size_x", ctypes.c_uint), ("size_y", ctypes.c_uint), ("n", ctypes.c_int)]


class Counters(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_ulonglong), ("out_of_grid", ctypes.c_ulonglong),
                ("bucket_overflow", ctypes.c_ulonglong), ("max_cell_occupancy", ctypes.c_uint),
                ("list_cap_risk", ctypes.c_uint)]


STATUS = {0: "SPH_OK", 1: "SPH_ERR_INVALID", 2: "SPH_ERR_CUDA", 3: "SPH_ERR_ALLOC",
          4: "SPH_ERR_CAPACITY", 5: "SPH_ERR_STATE", 6: "SPH_ERR_UNSUPPORTED"}


class SphError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class LatticeBlock(ctypes.Structure):
    """sph_lattice_block (include/sph_cuda.h)."""
    _fields_ = [("n", ctypes.c_int), ("cols", ctypes.c_int), ("x0", ctypes.c_double),
                ("y0", ctypes.c_double), ("spacing", ctypes.c_double), ("jitter", ctypes.c_double),
                ("seed", ctypes.c_ulonglong), ("counter0", ctypes.c_ulonglong)]


_lib = None

_P = ctypes.c_void_p
_SIGS = {
    "sph_cuda_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(Param), ctypes.POINTER(AABB),
                                       ctypes.POINTER(NeighborGrid), ctypes.c_int]),
    "sph_cuda_destroy": (ctypes.c_int, [_P]),
    "sph_cuda_create_ensemble": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(SceneDesc), ctypes.c_int,
                                                ctypes.c_int, ctypes.c_int]),
    "sph_render_liquid": (ctypes.c_int, [c_short_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "sph_cuda_render_liquid": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                              ctypes.c_void_p]),
    "sph_cuda_tunables_preset": (ctypes.c_int, [ctypes.POINTER(TunableParameters), ctypes.c_char]),
    "sph_cuda_mover_track": (ctypes.c_int, [ctypes.c_float, ctypes.c_float, c_float_p, c_int_p,
                                            c_float_p, c_float_p]),
    "sph_cuda_init_lattice": (ctypes.c_int, [_P, ctypes.POINTER(LatticeBlock), ctypes.c_int]),
    "sph_cuda_set_scene_params": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(TunableParameters)]),
    "sph_cuda_num_scenes": (ctypes.c_int, [_P]),
    "sph_cuda_scene_diagnostics": (ctypes.c_int, [_P, c_double_p]),
    "sph_cuda_set_launch_shapes": (ctypes.c_int, [_P, c_int_p]),
    "sph_cuda_get_launch_shapes": (ctypes.c_int, [_P, c_int_p]),
    "sph_cuda_autotune": (ctypes.c_int, [_P, ctypes.c_int, c_int_p]),
    "sph_cuda_set_long_row_masks": (ctypes.c_int, [_P, ctypes.c_int]),
    "sph_cuda_get_long_row_masks": (ctypes.c_int, [_P]),
    "sph_cuda_set_stream": (ctypes.c_int, [_P, _P]),
    "sph_cuda_upload": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.POINTER(FluidParticle)), ctypes.c_int]),
    "sph_cuda_upload_particles": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "sph_cuda_upload_soa": (ctypes.c_int, [_P, c_float_p, c_float_p, c_float_p, c_float_p, ctypes.c_int]),
    "sph_cuda_step": (ctypes.c_int, [_P, ctypes.POINTER(TunableParameters), ctypes.c_int]),
    "sph_cuda_step_schedule": (ctypes.c_int, [_P, ctypes.POINTER(TunableParameters), ctypes.c_int]),
    "sph_cuda_step_split": (ctypes.c_int, [_P, ctypes.POINTER(TunableParameters),
                                           ctypes.POINTER(TunableParameters)]),
    "sph_cuda_download": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.POINTER(FluidParticle)), ctypes.c_int]),
    "sph_cuda_download_particles": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "sph_cuda_download_soa": (ctypes.c_int, [_P] + [c_float_p] * 6 + [ctypes.c_int]),
    "sph_cuda_pack_coords_short": (ctypes.c_int, [_P, c_short_p, ctypes.c_int]),
    "sph_cuda_pack_coords_async": (ctypes.c_int, [_P, c_short_p, ctypes.c_int]),
    "sph_cuda_coords_wait": (ctypes.c_int, [_P, c_short_p]),
    "sph_cuda_rebuild_neighbors": (ctypes.c_int, [_P]),
    "sph_cuda_save_state": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "sph_cuda_load_state": (ctypes.c_int, [_P, ctypes.c_char_p]),
    "sph_cuda_synchronize": (ctypes.c_int, [_P]),
    "sph_cuda_get_counters": (ctypes.c_int, [_P, ctypes.POINTER(Counters)]),
    "sph_cuda_diagnostics": (ctypes.c_int, [_P, c_double_p]),
    "sph_cuda_neighbor_lists": (ctypes.c_int, [_P, c_int_p, c_int_p, ctypes.c_longlong,
                                               ctypes.POINTER(ctypes.c_longlong)]),
    "sph_cuda_probe_density": (ctypes.c_int, [_P, ctypes.POINTER(TunableParameters), c_float_p, c_float_p]),
    "sph_cuda_probe_relaxation": (ctypes.c_int, [_P, ctypes.POINTER(TunableParameters), c_float_p, c_float_p]),
    "sph_cuda_probe_viscosity": (ctypes.c_int, [_P, ctypes.POINTER(TunableParameters), c_float_p, c_float_p]),
    "sph_cuda_kernel_times": (ctypes.c_int, [_P, ctypes.POINTER(TunableParameters), c_float_p,
                                             ctypes.c_int, c_int_p]),
    "sph_cuda_kernel_name": (ctypes.c_char_p, [ctypes.c_int]),
    "sph_cuda_step_kernel_name": (ctypes.c_char_p, [_P, ctypes.c_int]),
    "sph_cuda_launches_per_step": (ctypes.c_int, [_P]),
    "sph_cuda_timer_start": (ctypes.c_int, [_P]),
    "sph_cuda_timer_stop": (ctypes.c_int, [_P, c_float_p]),
    "sph_cuda_host_alloc": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_size_t]),
    "sph_cuda_host_free": (ctypes.c_int, [_P]),
    "sph_cuda_debug_fail_allocation": (ctypes.c_int, [ctypes.c_int]),
    "sph_cuda_bounds_errors": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint)]),
    "sph_cuda_bounds_checked": (ctypes.c_int, []),
    "sph_cuda_last_error": (ctypes.c_char_p, []),
    "sph_cuda_abi_sizes": (ctypes.c_int, [c_int_p, ctypes.c_int]),
    # learned relaxation (include/sph_learned.h)
    "sph_learned_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_ulonglong]),
    "sph_learned_destroy": (ctypes.c_int, [_P]),
    "sph_learned_collect": (ctypes.c_int, [_P, _P, ctypes.c_float, c_int_p]),
    "sph_learned_num_samples": (ctypes.c_int, [_P]),
    "sph_learned_clear_samples": (ctypes.c_int, [_P]),
    "sph_learned_train": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, ctypes.c_float, c_float_p]),
    "sph_learned_calibrate": (ctypes.c_int, [_P, _P, ctypes.c_int, ctypes.c_float, c_float_p]),
    "sph_learned_num_params": (ctypes.c_int, []),
    "sph_learned_get_params": (ctypes.c_int, [_P, c_float_p]),
    "sph_learned_set_params": (ctypes.c_int, [_P, c_float_p]),
    "sph_learned_forward": (ctypes.c_int, [_P, c_float_p, ctypes.c_int, c_float_p]),
    "sph_learned_features": (ctypes.c_int, [_P, c_float_p, c_int_p]),
    "sph_learned_wait_selftest": (ctypes.c_int, [c_int_p]),
    "sph_learned_gemm_check": (ctypes.c_int, [c_float_p, c_float_p, c_float_p, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int]),
    "sph_cuda_set_learned": (ctypes.c_int, [_P, _P, ctypes.c_float]),
    "sph_cuda_learned_counts": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_ulonglong),
                                               ctypes.POINTER(ctypes.c_ulonglong)]),
}


def lib() -> ctypes.CDLL:
    """The loaded library.  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libsph_cuda is not built ({LIB_PATH} missing): run "
                              "`python -m sph_gb300.build` or __graft_entry__.build()")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(status: int) -> None:
    if status != 0:
        raise SphError(status, lib().sph_cuda_last_error().decode(errors="replace"))


def declared_symbols() -> list:
    """Every function name declared in include/*.h (for the export check)."""
    names = []
    for h in sorted(os.listdir(INCLUDE)):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(([^;{}]*)\)\s*;", text):
            name = m.group(1)
            prefix = text[max(0, m.start() - 80):m.start()]
            if "typedef" in prefix.split(";")[-1] or name in ("sizeof", "if", "while", "return"):
                continue
            names.append(name)
    return sorted(set(names))


def tunables(d: dict) -> TunableParameters:
    t = TunableParameters()
    for name, _ in TunableParameters._fields_:
        setattr(t, name, d[name])
    return t
