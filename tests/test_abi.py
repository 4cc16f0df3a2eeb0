"""Host-side checks of the C ABI: the library loads without a GPU, exports
every function its headers declare, and was compiled with the reference's
struct layouts.  No call here touches a GPU."""
import ctypes

import pytest

from sph_gb300 import _lib


def test_library_exports_every_declared_symbol(cuda_lib):
    declared = _lib.declared_symbols()
    assert "sph_cuda_step" in declared and "hash_fluid" in declared
    missing = [s for s in declared if not hasattr(cuda_lib, s)]
    assert not missing, missing


def test_struct_layouts_match_reference(cuda_lib):
    sizes = (ctypes.c_int * 7)()
    assert cuda_lib.sph_cuda_abi_sizes(sizes, 7) == 0
    expect = [ctypes.sizeof(_lib.FluidParticle), ctypes.sizeof(_lib.Neighbor),
              ctypes.sizeof(_lib.TunableParameters), ctypes.sizeof(_lib.Param),
              ctypes.sizeof(_lib.Bucket), ctypes.sizeof(_lib.NeighborGrid), ctypes.sizeof(_lib.AABB)]
    assert list(sizes) == expect
    assert list(sizes)[:4] == [52, 16, 64, 80] and list(sizes)[5:] == [40, 24]


def test_invalid_arguments_rejected_before_any_device_call(cuda_lib):
    h = ctypes.c_void_p()
    p = _lib.Param()
    b = _lib.AABB()
    g = _lib.NeighborGrid()  # spacing 0: invalid
    st = cuda_lib.sph_cuda_create(ctypes.byref(h), ctypes.byref(p), ctypes.byref(b), ctypes.byref(g), 10)
    assert st == 1 and not h.value
    assert b"grid" in cuda_lib.sph_cuda_last_error()
    g.spacing, g.size_x, g.size_y, g.max_bucket_size, g.max_neighbors = 1.0, 4, 4, 100, 400
    p.number_halo_particles = 3
    st = cuda_lib.sph_cuda_create(ctypes.byref(h), ctypes.byref(p), ctypes.byref(b), ctypes.byref(g), 10)
    assert st == 6 and b"halo" in cuda_lib.sph_cuda_last_error()
    assert cuda_lib.sph_cuda_step(None, None, 1) == 1


def test_kernel_names_without_gpu(cuda_lib):
    names = [cuda_lib.sph_cuda_kernel_name(k).decode() for k in range(11)]
    assert names[0] == "viscosity_predict" and "density" in names and "relax_update" in names


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libsph_cuda.so"))
    with pytest.raises(ImportError):
        _lib.lib()
