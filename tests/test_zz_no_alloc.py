"""The allocation-free density entry point, sph_cuda_density_static.

It serves callers that cannot call cudaMalloc (a loop inside another
framework's fixed device-memory budget, or one that cannot afford an
allocation's synchronisation): its scratch is one fixed-size device array
inside the library.  This test calls it through the C ABI on device buffers,
on consecutive calls with different states (so that contents left in the
shared array by one call cannot leak into the next), and checks it

* bit for bit against the allocating path (sph_cuda_probe_density): both
  run the same kernels on the same (cell, id) order;
* against the reference's own densities (golden vectors), per particle
  within 1e-5 relative;
* at the size limits (SPH_STATIC_MAX_PARTICLES particles on a grid of
  SPH_STATIC_MAX_CELLS cells, populated up to its last cells) with a few
  particles outside the grid, whose count the counters reader reports.

It lives in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

from conftest import bits_equal, golden, rel_ok
from sph_gb300 import Simulation, _lib, scenes

pytestmark = pytest.mark.gpu

MAX_N = 65536          # SPH_STATIC_MAX_PARTICLES
MAX_CELLS = 262144     # SPH_STATIC_MAX_CELLS


def _grid(config):
    g = _lib.NeighborGrid()
    g.spacing = config["spacing"]
    g.size_x, g.size_y = config["size_x"], config["size_y"]
    g.max_bucket_size, g.max_neighbors = config["max_bucket"], config["max_neighbors"]
    return g


@pytest.fixture
def lib(cuda_lib):
    f = cuda_lib.sph_cuda_density_static
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_lib.NeighborGrid),
                  ctypes.POINTER(_lib.TunableParameters), ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p]
    c = cuda_lib.sph_cuda_density_static_counters
    c.restype = ctypes.c_int
    c.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    return cuda_lib


def _density_static(lib, torch, x, y, config, params):
    """One call on device buffers; returns (rho, rho_near, counters)."""
    dev = torch.device("cuda:0")
    tx = torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(dev)
    ty = torch.from_numpy(np.ascontiguousarray(y, np.float32)).to(dev)
    rho = torch.full((len(x),), -1.0, dtype=torch.float32, device=dev)
    rhon = torch.full((len(x),), -1.0, dtype=torch.float32, device=dev)
    cnt = torch.zeros(ctypes.sizeof(_lib.Counters), dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    fp = ctypes.c_void_p
    st = lib.sph_cuda_density_static(fp(tx.data_ptr()), fp(ty.data_ptr()), len(x),
                                     ctypes.byref(_grid(config)), ctypes.byref(_lib.tunables(params)),
                                     fp(rho.data_ptr()), fp(rhon.data_ptr()), None)
    _lib.check(st)
    _lib.check(lib.sph_cuda_density_static_counters(fp(cnt.data_ptr()), None))
    torch.cuda.synchronize()
    c = _lib.Counters.from_buffer_copy(cnt.cpu().numpy().tobytes())
    return rho.cpu().numpy(), rhon.cpu().numpy(), {k: getattr(c, k) for k, _ in _lib.Counters._fields_}


def _allocating(x, y, config, params):
    with Simulation(params, config, len(x)) as s:
        s.upload(x, y)
        rho, rhon = s.probe_density(params)
    return rho, rhon


def test_density_static_matches_allocating_path_and_reference(lib):
    torch = pytest.importorskip("torch")
    g = golden("cfg1")
    sc = scenes.config1()
    P, C = sc.params.as_dict(), sc.config()
    for t in (100, 1000, 100):  # calls in a row, different states, then the first again
        x, y = g[f"s{t}_x"], g[f"s{t}_y"]
        rho, rhon, cnt = _density_static(lib, torch, x, y, C, P)
        ref_rho, ref_rhon = _allocating(x, y, C, P)
        assert bits_equal(rho, ref_rho) and bits_equal(rhon, ref_rhon), t
        for got, want in ((rho, g[f"h{t}_rho"]), (rhon, g[f"h{t}_rhon"])):
            ok, err = rel_ok(got, want)
            assert ok, (t, err)
        assert cnt["out_of_grid"] == 0 and cnt["bucket_overflow"] == 0


def _limit_case():
    """SPH_STATIC_MAX_PARTICLES particles on a 512 x 512 grid (h = 1): a
    jittered 0.5h lattice filling the top-right 128 x 128 cells (so the last
    cells and the last words of the no-cell bitmap are in use), with eight
    of the lattice points moved outside the grid: four below or left of it,
    two at y == size_y (the first row past the grid), and two at
    x == size_x, which alias to the first cell of the next row, as
    hash_val does (hash.c:35-47)."""
    side = 256
    i = np.arange(side * side)
    rng = np.random.default_rng(1234)
    x = (384.0 + 0.25 + 0.5 * (i % side) + rng.uniform(-0.05, 0.05, i.size)).astype(np.float32)
    y = (384.0 + 0.25 + 0.5 * (i // side) + rng.uniform(-0.05, 0.05, i.size)).astype(np.float32)
    outside = [(-1.0, 400.0), (450.0, -0.5), (-3.0, -3.0), (-0.25, 511.0),
               (450.0, 512.0), (500.5, 512.0)]
    for k, (ox, oy) in enumerate(outside):
        x[17 * k + 5], y[17 * k + 5] = ox, oy
    x[7000], y[7000] = 512.0, 400.5
    x[9000], y[9000] = 512.0, 300.5
    config = dict(box=(0.0, 512.0, 0.0, 512.0), spacing=1.0, size_x=512, size_y=512,
                  max_bucket=100, max_neighbors=400)
    return x, y, config, len(outside)


def test_density_static_at_the_size_limits(lib):
    torch = pytest.importorskip("torch")
    x, y, config, n_out = _limit_case()
    assert len(x) == MAX_N and config["size_x"] * config["size_y"] == MAX_CELLS
    P = scenes.config1().params.as_dict()
    for _ in range(2):  # twice in a row: the second call starts from the first's leftovers
        rho, rhon, cnt = _density_static(lib, torch, x, y, config, P)
        ref_rho, ref_rhon = _allocating(x, y, config, P)
        assert bits_equal(rho, ref_rho) and bits_equal(rhon, ref_rhon)
        assert cnt["out_of_grid"] == n_out
        assert cnt["bucket_overflow"] == 0 and 1 <= cnt["max_cell_occupancy"] <= 12
        assert (rho > 0).sum() > MAX_N - 64  # a dense block: nearly every particle has neighbours


def test_density_static_rejects_oversize(lib):
    sc = scenes.config1()
    g = _grid(sc.config())
    t = _lib.tunables(sc.params.as_dict())
    st = lib.sph_cuda_density_static(None, None, MAX_N + 1, ctypes.byref(g), ctypes.byref(t), None, None, None)
    assert st == 4 and b"at most 65536" in lib.sph_cuda_last_error()
    g.size_x, g.size_y = 1024, 1024
    st = lib.sph_cuda_density_static(None, None, 10, ctypes.byref(g), ctypes.byref(t), None, None, None)
    assert st == 4 and b"cells" in lib.sph_cuda_last_error()
    assert lib.sph_cuda_density_static_counters(None, None) == 1
