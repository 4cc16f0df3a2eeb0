"""CPU oracle for the SPH compute step -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package.  It is the checker, never the thing measured or shipped:
the product library (sph_gb300 / libsph_cuda) does not import it and has no
CPU fallback.

Two back ends with one Python interface (`Sim`):

* "ref"  -- oracle/_ref/libsph_ref.so: the reference's own src/hash.c and
  src/fluid.c, compiled unmodified by `make -C oracle ref` where the
  reference sources exist.  Absent elsewhere (e.g. on an Arm GPU host).
* "port" -- oracle/libsph_oracle.so: the C restatement (sph_oracle.c), pinned
  bit-exactly to "ref" and to the committed golden vectors; it also carries
  the FP64 gather oracles and the float Jacobi step.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "libsph_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsph_ref.so")
REF_FASTMATH_LIB = os.path.join(HERE, "_ref", "libsph_ref_fastmath.so")
# Where the reference's src/ lies: $SPH_REF_SRC, else a checkout named
# "reference" beside this repository.  Absent (as on a machine that only
# runs the GPU tests), the "ref" back end is simply not built.
REF_SRC = os.environ.get("SPH_REF_SRC") or os.path.join(
    os.path.dirname(os.path.dirname(HERE)), "reference", "src")

FIELDS = ("x_prev", "y_prev", "x", "y", "v_x", "v_y", "a_x", "a_y", "density",
          "density_near", "pressure", "pressure_near")


class Tunables(ctypes.Structure):
    """Layout of the reference's tunable_parameters (fluid.h:78-97)."""
    _fields_ = [(n, ctypes.c_float) for n in (
        "rest_density", "smoothing_radius", "g", "k", "k_near", "k_spring", "sigma", "beta",
        "time_step", "node_start_x", "node_end_x", "mover_center_x", "mover_center_y",
        "mover_width", "mover_height")] + [
        ("mover_type", ctypes.c_byte), ("kill_sim", ctypes.c_byte), ("active", ctypes.c_byte)]


class SimConfig(ctypes.Structure):
    _fields_ = [("box", ctypes.c_float * 4), ("spacing", ctypes.c_float),
                ("size_x", ctypes.c_int), ("size_y", ctypes.c_int),
                ("max_bucket", ctypes.c_int), ("max_neighbors", ctypes.c_int)]


def tunables_from(d: dict) -> Tunables:
    t = Tunables()
    for name, _ in Tunables._fields_:
        setattr(t, name, d[name])
    return t


def config_from(d: dict) -> SimConfig:
    c = SimConfig()
    c.box[:] = list(d["box"])
    c.spacing = d["spacing"]
    c.size_x, c.size_y = d["size_x"], d["size_y"]
    c.max_bucket, c.max_neighbors = d["max_bucket"], d["max_neighbors"]
    return c


def build(ref: bool | None = None) -> None:
    """Compile the restatement; also the reference when its sources exist."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_SRC={REF_SRC}"], check=True)


def ref_available(fastmath: bool = False) -> bool:
    return os.path.exists(REF_FASTMATH_LIB if fastmath else REF_LIB)


_libs: dict = {}

_P = ctypes.c_void_p
_F = ctypes.POINTER(ctypes.c_float)
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def _load(kind: str):
    if kind in _libs:
        return _libs[kind]
    path = {"port": PORT_LIB, "ref": REF_LIB, "ref_fastmath": REF_FASTMATH_LIB}[kind]
    if not os.path.exists(path):
        raise FileNotFoundError(f"oracle library {path} not built (make -C oracle"
                                f"{'' if kind == 'port' else ' ref'})")
    lib = ctypes.CDLL(path)
    pre = "orc_" if kind == "port" else "ref_"
    f = lambda n: getattr(lib, pre + n)  # noqa: E731
    f("create").restype = _P
    f("create").argtypes = [ctypes.c_int, _F, _F, _F, _F, ctypes.POINTER(Tunables),
                            ctypes.POINTER(SimConfig)]
    f("destroy").argtypes = [_P]
    f("set_tunables").argtypes = [_P, ctypes.POINTER(Tunables)]
    f("step").argtypes = [_P, ctypes.c_int, _F, _D]
    f("get").argtypes = [_P, _F]
    f("set_state").argtypes = [_P, _F, _F, _F, _F]
    f("call").argtypes = [_P, ctypes.c_int]
    f("pack_coords").argtypes = [_P, ctypes.POINTER(ctypes.c_short)]
    if kind == "port":
        lib.orc_hash.argtypes = [_P, ctypes.c_int]
        lib.orc_hash_fresh.argtypes = [_P, ctypes.c_int]
        lib.orc_get_lists.restype = ctypes.c_long
        lib.orc_get_lists.argtypes = [_P, _I, _I, ctypes.c_long]
        lib.orc_set_lists.argtypes = [_P, _I, _I]
        lib.orc_density_f64.argtypes = [_P, _D, _D]
        lib.orc_relax_f64.argtypes = [_P, _F, _F, _D, _D, _D]
        lib.orc_viscosity_f64.argtypes = [_P, _D, _D, _D]
        lib.orc_step_jacobi.argtypes = [_P, ctypes.c_int, _F, _D]
        lib.orc_step_jacobi_split.argtypes = [_P, ctypes.POINTER(Tunables), ctypes.POINTER(Tunables)]
        lib.orc_diagnostics.argtypes = [_P, _D]
        lib.orc_cell_key.restype = ctypes.c_uint
        lib.orc_cell_key.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.POINTER(SimConfig)]
    else:
        lib.ref_hash.restype = ctypes.c_int
        lib.ref_hash.argtypes = [_P, ctypes.c_int, _I, _I, ctypes.c_int]
        lib.ref_hash_val.restype = ctypes.c_uint
        lib.ref_hash_val.argtypes = [_P, ctypes.c_float, ctypes.c_float]
    _libs[kind] = lib
    return lib


def _fp(a):
    return a.ctypes.data_as(_F) if a is not None else None


def _dp(a):
    return a.ctypes.data_as(_D) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(_I)


class Sim:
    """One single-domain simulation on the CPU oracle.

    kind: "port" (the restatement), "ref" or "ref_fastmath" (the reference's
    compiled step functions).  Particle i has id i throughout."""

    def __init__(self, kind: str, x, y, vx, vy, params: dict, config: dict):
        self.kind = kind
        self.lib = _load(kind)
        self.pre = "orc_" if kind == "port" else "ref_"
        self.n = int(len(x))
        self._keep = [np.ascontiguousarray(a, np.float32) for a in (x, y, vx, vy)]
        self.tun = tunables_from(params)
        self.cfg = config_from(config)
        self.max_neighbors = int(config["max_neighbors"])
        self.h = self._f("create")(self.n, *[_fp(a) for a in self._keep], ctypes.byref(self.tun),
                                   ctypes.byref(self.cfg))
        if not self.h:
            raise MemoryError("oracle create failed")

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    def close(self):
        if getattr(self, "h", None):
            self._f("destroy")(self.h)
            self.h = None

    __del__ = close

    def set_params(self, params: dict):
        self.tun = tunables_from(params)
        self._f("set_tunables")(self.h, ctypes.byref(self.tun))

    def set_state(self, x, y, vx=None, vy=None):
        arrs = [None if a is None else np.ascontiguousarray(a, np.float32) for a in (x, y, vx, vy)]
        self._f("set_state")(self.h, *[_fp(a) for a in arrs])

    def step(self, nsteps: int, mover_xy=None, jacobi: bool = False) -> np.ndarray:
        """Runs nsteps; returns per-step diagnostics [nsteps, 3] (mean density,
        mean near density, kinetic energy per particle)."""
        diag = np.zeros((nsteps, 3), np.float64)
        mv = None if mover_xy is None else np.ascontiguousarray(mover_xy, np.float32).reshape(-1)
        if jacobi:
            if self.kind != "port":
                raise ValueError("the Jacobi step exists only in the restatement")
            self.lib.orc_step_jacobi(self.h, nsteps, _fp(mv), _dp(diag))
        else:
            self._f("step")(self.h, nsteps, _fp(mv), _dp(diag))
        return diag

    def step_jacobi_split(self, before: dict | None, after: dict):
        """One float Jacobi step with the tunables switched after
        predict_positions (fluid.c:293-294); `after` stays in force."""
        if self.kind != "port":
            raise ValueError("the Jacobi step exists only in the restatement")
        b = None if before is None else ctypes.byref(tunables_from(before))
        self.tun = tunables_from(after)
        self.lib.orc_step_jacobi_split(self.h, b, ctypes.byref(self.tun))

    def get(self) -> dict:
        out = np.zeros((self.n, 12), np.float32)
        self._f("get")(self.h, _fp(out))
        return {k: out[:, i].copy() for i, k in enumerate(FIELDS)}

    def call(self, which: int):
        """0 gravity, 1 viscosity, 2 predict, 3 relaxation, 4 velocity update."""
        self._f("call")(self.h, which)

    def pack_coords(self) -> np.ndarray:
        out = np.zeros((self.n, 2), np.int16)
        self._f("pack_coords")(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_short)))
        return out

    def hash(self, compute_density: bool = True):
        """Runs the hash on the current positions (densities zeroed first when
        compute_density).  Returns (counts[n], ids[total]) of the half lists."""
        counts = np.zeros(self.n, np.int32)
        cap = self.n * self.max_neighbors
        ids = np.zeros(max(cap, 1), np.int32)
        if self.kind == "port":
            self.lib.orc_hash_fresh(self.h, int(compute_density))
            total = self.lib.orc_get_lists(self.h, _ip(counts), _ip(ids), cap)
        else:
            total = self.lib.ref_hash(self.h, int(compute_density), _ip(counts), _ip(ids), cap)
        if total < 0:
            raise RuntimeError("neighbour list buffer too small")
        return counts, ids[:total].copy()

    # ---- FP64 gather oracles (restatement only) ----
    def set_lists(self, counts, ids):
        self.lib.orc_set_lists(self.h, _ip(np.ascontiguousarray(counts, np.int32)),
                               _ip(np.ascontiguousarray(ids, np.int32)))

    def density_f64(self):
        rho = np.zeros(self.n, np.float64)
        rhon = np.zeros(self.n, np.float64)
        self.lib.orc_density_f64(self.h, _dp(rho), _dp(rhon))
        return rho, rhon

    def relax_f64(self, rho, rhon):
        rho = np.ascontiguousarray(rho, np.float32)
        rhon = np.ascontiguousarray(rhon, np.float32)
        dx, dy, sc = (np.zeros(self.n, np.float64) for _ in range(3))
        self.lib.orc_relax_f64(self.h, _fp(rho), _fp(rhon), _dp(dx), _dp(dy), _dp(sc))
        return dx, dy, sc

    def viscosity_f64(self):
        dx, dy, sc = (np.zeros(self.n, np.float64) for _ in range(3))
        self.lib.orc_viscosity_f64(self.h, _dp(dx), _dp(dy), _dp(sc))
        return dx, dy, sc


def cell_key(x: float, y: float, config: dict) -> int:
    """hash_val (hash.c:35-47) restated; 0xFFFFFFFF for out-of-grid points."""
    lib = _load("port")
    return int(lib.orc_cell_key(ctypes.c_float(x), ctypes.c_float(y), ctypes.byref(config_from(config))))


def pair_set(counts, ids) -> np.ndarray:
    """Unordered pair set {min(i,j), max(i,j)} of half lists, as sorted int64 keys."""
    owner = np.repeat(np.arange(len(counts), dtype=np.int64), counts)
    other = ids.astype(np.int64)
    lo, hi = np.minimum(owner, other), np.maximum(owner, other)
    return np.unique(lo * (1 << 32) + hi)
