"""The allocation-free density entry point, sph_cuda_density_static.

It serves callers that cannot call cudaMalloc (a loop inside another
framework's fixed device-memory budget, or one that cannot afford an
allocation's synchronisation): its scratch is one fixed-size device array
inside the library.  This test calls it through the C ABI on device buffers
and checks it against the allocating path (sph_cuda_probe_density) on two
consecutive calls, the second on a different state, so that contents left
in the shared array by the first call cannot leak into the second.  It
lives in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden
from sph_gb300 import Simulation, _lib, scenes

pytestmark = pytest.mark.gpu


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
    return cuda_lib


def _density_static(lib, torch, x, y, config, params):
    dev = torch.device("cuda:0")
    tx = torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(dev)
    ty = torch.from_numpy(np.ascontiguousarray(y, np.float32)).to(dev)
    rho = torch.full((len(x),), -1.0, dtype=torch.float32, device=dev)
    rhon = torch.full((len(x),), -1.0, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    fp = ctypes.c_void_p
    st = lib.sph_cuda_density_static(fp(tx.data_ptr()), fp(ty.data_ptr()), len(x),
                                     ctypes.byref(_grid(config)), ctypes.byref(_lib.tunables(params)),
                                     fp(rho.data_ptr()), fp(rhon.data_ptr()), None)
    _lib.check(st)
    torch.cuda.synchronize()
    return rho.cpu().numpy(), rhon.cpu().numpy()


def test_density_static_matches_allocating_path(lib):
    torch = pytest.importorskip("torch")
    g = golden("cfg1")
    sc = scenes.config1()
    P, C = sc.params.as_dict(), sc.config()
    for t in (100, 1000):  # two calls in a row, different states
        x, y = g[f"s{t}_x"], g[f"s{t}_y"]
        rho, rhon = _density_static(lib, torch, x, y, C, P)
        with Simulation(P, C, sc.n) as s:
            s.upload(x, y)
            ref_rho, ref_rhon = s.probe_density(P)
        assert np.allclose(rho, ref_rho, rtol=1e-5, atol=1e-7), t
        assert np.allclose(rhon, ref_rhon, rtol=1e-5, atol=1e-7), t


def test_density_static_rejects_oversize(lib):
    sc = scenes.config1()
    g = _grid(sc.config())
    t = _lib.tunables(sc.params.as_dict())
    st = lib.sph_cuda_density_static(None, None, 65537, ctypes.byref(g), ctypes.byref(t), None, None, None)
    assert st == 4 and b"at most 65536" in lib.sph_cuda_last_error()
    g.size_x, g.size_y = 1024, 1024
    st = lib.sph_cuda_density_static(None, None, 10, ctypes.byref(g), ctypes.byref(t), None, None, None)
    assert st == 4 and b"cells" in lib.sph_cuda_last_error()
