"""The reference-named entry points (include/sph_legacy.h), called through
the C ABI on the reference's own structs, against the reference's outputs
(golden vectors), the restatement that is pinned to it, and the FP64 gather
oracle for the two pair passes."""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import EDGE_CONFIG, bits_equal, golden, rel_ok
from sph_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

FP = ctypes.POINTER(_lib.FluidParticle)


class Host:
    """The reference's host-side state: particle array, pointer array,
    neighbour lists and grid buckets, as fluid.c:178-225 allocates them."""

    def __init__(self, state: dict, config: dict, params: dict):
        n = len(state["x"])
        self.n = n
        self.parts = (_lib.FluidParticle * n)()
        for i in range(n):
            p = self.parts[i]
            for k, v in state.items():
                setattr(p, k, float(v[i]))
            p.id = i
        self.ptrs = (FP * n)(*[ctypes.pointer(self.parts[i]) for i in range(n)])
        mn, mb = config["max_neighbors"], config["max_bucket"]
        cells = config["size_x"] * config["size_y"]
        self.nstore = (FP * (n * mn))()
        self.nbrs = (_lib.Neighbor * n)()
        base = ctypes.addressof(self.nstore)
        for i in range(n):
            self.nbrs[i].fluid_neighbors = ctypes.cast(base + i * mn * ctypes.sizeof(FP), ctypes.POINTER(FP))
        self.bstore = (FP * (cells * mb))()
        self.buckets = (_lib.Bucket * cells)()
        bb = ctypes.addressof(self.bstore)
        for c in range(cells):
            self.buckets[c].fluid_particles = ctypes.cast(bb + c * mb * ctypes.sizeof(FP), ctypes.POINTER(FP))
        self.grid = _lib.NeighborGrid()
        self.grid.spacing = config["spacing"]
        self.grid.size_x, self.grid.size_y = config["size_x"], config["size_y"]
        self.grid.max_neighbors, self.grid.max_bucket_size = mn, mb
        self.grid.neighbors = self.nbrs
        self.grid.grid_buckets = self.buckets
        self.param = _lib.Param()
        self.param.tunable_params = _lib.tunables(params)
        self.param.number_fluid_particles_global = n
        self.param.number_fluid_particles_local = n
        self.param.max_fluid_particle_index = n - 1
        self.box = _lib.AABB()
        self.box.min_x, self.box.max_x, self.box.min_y, self.box.max_y = config["box"]
        self.base = ctypes.addressof(self.parts)

    def field(self, name):
        return np.array([getattr(self.parts[i], name) for i in range(self.n)], np.float32)

    def lists(self):
        counts = np.array([self.nbrs[i].number_fluid_neighbors for i in range(self.n)], np.int32)
        ids = [self.nbrs[i].fluid_neighbors[k].contents.id for i in range(self.n) for k in range(counts[i])]
        return counts, np.array(ids, np.int32)

    def set_lists(self, counts, ids):
        o = 0
        for i in range(self.n):
            self.nbrs[i].number_fluid_neighbors = int(counts[i])
            for k in range(counts[i]):
                self.nbrs[i].fluid_neighbors[k] = self.ptrs[int(ids[o + k])]
            o += counts[i]


@pytest.fixture(scope="module")
def L(cuda_lib):
    l = cuda_lib
    sigs = {
        "apply_gravity": [ctypes.c_void_p, ctypes.POINTER(_lib.Param)],
        "predict_positions": [ctypes.c_void_p, ctypes.POINTER(_lib.AABB), ctypes.POINTER(_lib.Param)],
        "updateVelocities": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(_lib.AABB), ctypes.POINTER(_lib.Param)],
        "viscosity_impluses": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(_lib.Param)],
        "double_density_relaxation": [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(_lib.Param)],
        "hash_fluid": [ctypes.c_void_p, ctypes.POINTER(_lib.NeighborGrid), ctypes.POINTER(_lib.Param), ctypes.c_bool],
        "hash_halo": [ctypes.c_void_p, ctypes.POINTER(_lib.NeighborGrid), ctypes.POINTER(_lib.Param), ctypes.c_bool],
        "identify_oob_particles": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(_lib.AABB),
                                   ctypes.POINTER(_lib.Param)],
        "boundaryConditions": [FP, ctypes.POINTER(_lib.AABB), ctypes.POINTER(_lib.Param)],
        "updateVelocity": [FP, ctypes.POINTER(_lib.Param)],
        "checkVelocity": [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
        "calculate_density": [FP, FP, ctypes.c_float],
        "hash_val": [ctypes.c_float, ctypes.c_float, ctypes.POINTER(_lib.NeighborGrid), ctypes.POINTER(_lib.Param)],
    }
    for name, args in sigs.items():
        getattr(l, name).argtypes = args
        getattr(l, name).restype = None
    l.hash_val.restype = ctypes.c_uint
    l.sph_legacy_status.restype = ctypes.c_int
    return l


def state_of(g, t):
    st = {k: g[f"s{t}_{k}"] for k in ("x", "y", "v_x", "v_y", "density", "density_near")}
    st["x_prev"], st["y_prev"] = st["x"], st["y"]
    return st


def cfg1():
    sc = scenes.config1()
    return sc, sc.params.as_dict(), sc.config()


def test_apply_gravity_bit_exact(L):
    g = golden("cfg1")
    sc, P, C = cfg1()
    st = state_of(g, 10)
    h = Host(st, C, P)
    L.apply_gravity(h.ptrs, ctypes.byref(h.param))
    assert L.sph_legacy_status() == 0
    port = oracle.Sim("port", st["x"], st["y"], st["v_x"], st["v_y"], P, C)
    port.call(0)
    s = port.get()
    assert bits_equal(h.field("v_y"), s["v_y"]) and not h.field("density").any()


@pytest.mark.parametrize("tag", ["sphere", "rect"])
def test_predict_positions_matches_reference(L, tag):
    g = golden("predict")
    w, hh, cx, cy, dt = (float(v) for v in g[f"{tag}_params"])
    p = scenes.Params(mover_type=scenes.SPHERE_MOVER if tag == "sphere" else scenes.RECTANGLE_MOVER,
                      mover_width=w, mover_height=hh, mover_center_x=cx, mover_center_y=cy, time_step=dt)
    st = dict(x=g["x"], y=g["y"], v_x=g["vx"], v_y=g["vy"])
    h = Host(st, EDGE_CONFIG, p.as_dict())
    L.predict_positions(h.ptrs, ctypes.byref(h.box), ctypes.byref(h.param))
    assert L.sph_legacy_status() == 0
    assert bits_equal(h.field("x"), g[f"{tag}_x"]) and bits_equal(h.field("y"), g[f"{tag}_y"])
    assert bits_equal(h.field("x_prev"), g["x"])


def test_update_velocities_bit_exact(L):
    g = golden("cfg1")
    sc, P, C = cfg1()
    st = state_of(g, 100)
    st["x_prev"] = g["s10_x"]
    st["y_prev"] = g["s10_y"]
    h = Host(st, C, P)
    L.updateVelocities(h.ptrs, None, ctypes.byref(h.box), ctypes.byref(h.param))
    port = oracle.Sim("port", g["s10_x"], g["s10_y"], st["v_x"], st["v_y"], P, C)
    port.call(2)  # x_prev = x (s10)
    port.set_state(st["x"], st["y"])
    port.call(4)
    s = port.get()
    for k in ("x", "y", "v_x", "v_y"):
        assert bits_equal(h.field(k), s[k]), k


@pytest.mark.parametrize("t", [100, 1000])
def test_hash_fluid_lists_buckets_density(L, t):
    g = golden("cfg1")
    sc, P, C = cfg1()
    st = state_of(g, t)
    st["density"] = np.zeros_like(st["x"])
    st["density_near"] = np.zeros_like(st["x"])
    h = Host(st, C, P)
    L.hash_fluid(h.ptrs, ctypes.byref(h.grid), ctypes.byref(h.param), True)
    assert L.sph_legacy_status() == 0
    counts, ids = h.lists()
    assert np.array_equal(counts, g[f"h{t}_counts"]) and np.array_equal(ids, g[f"h{t}_ids"])
    rho = h.field("density")
    ok, err = rel_ok(rho, g[f"h{t}_rho"])
    assert ok, err
    ok, err = rel_ok(h.field("density_near"), g[f"h{t}_rhon"])
    assert ok, err
    # buckets: each cell's members in id order (hash.c:153-163)
    keys = np.array([oracle.cell_key(float(x), float(y), C) for x, y in zip(st["x"], st["y"])])
    for c in np.unique(keys)[:200]:
        b = h.buckets[int(c)]
        got = [b.fluid_particles[k].contents.id for k in range(b.number_fluid)]
        assert got == sorted(np.nonzero(keys == c)[0].tolist())[:100]


def test_viscosity_impluses_fp64(L):
    g = golden("cfg1")
    sc, P, C = cfg1()
    st = state_of(g, 100)
    h = Host(st, C, P)
    h.set_lists(g["h100_counts"], g["h100_ids"])
    L.viscosity_impluses(h.ptrs, h.nbrs, ctypes.byref(h.param))
    assert L.sph_legacy_status() == 0
    orc = oracle.Sim("port", st["x"], st["y"], st["v_x"], st["v_y"], P, C)
    orc.set_lists(g["h100_counts"], g["h100_ids"])
    dvx, dvy, scale = orc.viscosity_f64()
    for k, d in (("v_x", dvx), ("v_y", dvy)):
        err = np.abs(h.field(k).astype(np.float64) - (st[k].astype(np.float64) + d))
        assert np.all(err <= 1e-5 * scale + 2 * np.spacing(np.abs(st[k]) + 1e-3)), k


def test_double_density_relaxation_fp64(L):
    g = golden("cfg1")
    sc, P, C = cfg1()
    st = state_of(g, 100)
    st["density"], st["density_near"] = g["h100_rho"], g["h100_rhon"]
    h = Host(st, C, P)
    h.set_lists(g["h100_counts"], g["h100_ids"])
    L.double_density_relaxation(h.ptrs, h.nbrs, ctypes.byref(h.param))
    assert L.sph_legacy_status() == 0
    orc = oracle.Sim("port", st["x"], st["y"], st["v_x"], st["v_y"], P, C)
    orc.set_lists(g["h100_counts"], g["h100_ids"])
    dx, dy, scale = orc.relax_f64(st["density"], st["density_near"])
    for k, d in (("x", dx), ("y", dy)):
        err = np.abs(h.field(k).astype(np.float64) - (st[k].astype(np.float64) + d))
        assert np.all(err <= 1e-5 * scale + 2 * np.spacing(np.abs(st[k]))), k
    k32, r32 = np.float32(P["k"]), np.float32(P["rest_density"])
    assert bits_equal(h.field("pressure"), k32 * (st["density"] - r32))
    assert bits_equal(h.field("pressure_near"), np.float32(P["k_near"]) * st["density_near"])


def test_single_particle_functions(L):
    g = golden("predict")
    w, hh, cx, cy, dt = (float(v) for v in g["rect_params"])
    p = scenes.Params(mover_type=scenes.RECTANGLE_MOVER, mover_width=w, mover_height=hh,
                      mover_center_x=cx, mover_center_y=cy, time_step=dt).as_dict()
    h = Host(dict(x=g["x"][:64], y=g["y"][:64], v_x=g["vx"][:64], v_y=g["vy"][:64]), EDGE_CONFIG, p)
    dt32 = np.float32(dt)
    for i in range(64):
        part = h.parts[i]
        part.x = float(np.float32(g["x"][i]) + np.float32(g["vx"][i]) * dt32)
        part.y = float(np.float32(g["y"][i]) + np.float32(g["vy"][i]) * dt32)
        L.boundaryConditions(ctypes.pointer(part), ctypes.byref(h.box), ctypes.byref(h.param))
        assert part.x == g["rect_x"][i] and part.y == g["rect_y"][i]
    # updateVelocity: v = (x - x_prev)/dt clamped (no boundary conditions)
    part = h.parts[0]
    part.x, part.y, part.x_prev, part.y_prev = 3.0, 4.0, 2.9, 4.5
    L.updateVelocity(ctypes.pointer(part), ctypes.byref(h.param))
    assert part.v_x == np.float32((np.float32(3.0) - np.float32(2.9)) / dt32) and part.v_y == -5.0
    vx, vy = ctypes.c_float(7.5), ctypes.c_float(-0.25)
    L.checkVelocity(ctypes.byref(vx), ctypes.byref(vy))
    assert (vx.value, vy.value) == (5.0, -0.25)
    a, b = h.parts[1], h.parts[2]
    a.density = b.density = 1.0
    a.density_near = b.density_near = 0.5
    L.calculate_density(ctypes.pointer(a), ctypes.pointer(b), 0.25)
    assert a.density == b.density == np.float32(1.0) + np.float32(0.75) * np.float32(0.75)
    L.calculate_density(ctypes.pointer(a), ctypes.pointer(b), 1.0)  # r == h: nothing
    assert a.density == np.float32(1.5625)
    # hash_val, including the right-wall aliasing of hash.c:41-44
    grid = h.grid
    assert L.hash_val(3.5, 2.25, ctypes.byref(grid), ctypes.byref(h.param)) == 2 * 16 + 3
    assert L.hash_val(16.0, 9.3, ctypes.byref(grid), ctypes.byref(h.param)) == 10 * 16 + 0
    assert L.hash_val(-0.5, 1.0, ctypes.byref(grid), ctypes.byref(h.param)) == 0xFFFFFFFF
    assert L.sph_legacy_status() == 0


def test_single_domain_halo_and_oob(L):
    g = golden("cfg1")
    sc, P, C = cfg1()
    st = state_of(g, 100)
    h = Host(st, C, P)
    L.hash_halo(h.ptrs, ctypes.byref(h.grid), ctypes.byref(h.param), True)
    assert L.sph_legacy_status() == 0
    L.identify_oob_particles(h.ptrs, None, None, ctypes.byref(h.box), ctypes.byref(h.param))
    assert L.sph_legacy_status() == 0
    h.parts[5].x = 200.0
    L.identify_oob_particles(h.ptrs, None, None, ctypes.byref(h.box), ctypes.byref(h.param))
    assert L.sph_legacy_status() == 6
    h.param.number_halo_particles = 4
    L.hash_halo(h.ptrs, ctypes.byref(h.grid), ctypes.byref(h.param), True)
    assert L.sph_legacy_status() == 6
