"""Live tunables: the render rank's fluid presets and its inactive-mode
mover path, as host helpers of the C ABI (no GPU needed)."""
import ctypes

import numpy as np
import pytest

from sph_gb300 import _lib, scenes


def test_presets(cuda_lib):
    tp = _lib.tunables(scenes.Params().as_dict())
    expect = {  # controls.c:344-401
        b"x": (6.0, 0.2, 6.0, 10.0, 5.0, 0.5, 30.0),
        b"y": (6.0, 0.1, 3.0, -30.0, 100.0, 10.0, 30.0),
        b"a": (0.0, 0.2, 6.0, 10.0, 20.0, 2.0, 55.0),
        b"b": (6.0, 0.0, 0.0, 115.0, 20.0, 2.0, 0.0),
    }
    for k, v in expect.items():
        assert cuda_lib.sph_cuda_tunables_preset(ctypes.byref(tp), k) == 0
        got = (tp.g, tp.k, tp.k_near, tp.k_spring, tp.sigma, tp.beta, tp.rest_density)
        assert np.allclose(got, v, rtol=0, atol=1e-7), k
    tp.mover_width = tp.mover_height = 7.0
    assert cuda_lib.sph_cuda_tunables_preset(ctypes.byref(tp), b"m") == 0
    assert tp.mover_width == 2.0 and tp.mover_height == 2.0
    assert cuda_lib.sph_cuda_tunables_preset(ctypes.byref(tp), b"q") != 0


def test_mover_path(cuda_lib):
    gx, d = ctypes.c_float(0.0), ctypes.c_int(1)
    cx, cy = ctypes.c_float(), ctypes.c_float()
    xs, ys, dirs = [], [], []
    for _ in range(450):
        assert cuda_lib.sph_cuda_mover_track(ctypes.c_float(15.0), ctypes.c_float(8.4375),
                                             ctypes.byref(gx), ctypes.byref(d),
                                             ctypes.byref(cx), ctypes.byref(cy)) == 0
        xs.append(cx.value)
        ys.append(cy.value)
        dirs.append(d.value)
    # restatement of renderer.c:493-532 in float32
    g, dd = np.float32(0.0), 1
    for i in range(450):
        g = np.float32(g + np.float32(0.01) * np.float32(dd))
        if g > 1.0 or g < -1.0:
            dd = -dd
        gy = np.float32(np.sin(np.float32(3.14) * np.float32(5.0) * g) / np.float32(10.0) - np.float32(0.6))
        assert abs(xs[i] - (g * 7.5 + 7.5)) < 1e-5
        assert abs(ys[i] - (gy * np.float32(4.21875) + np.float32(4.21875))) < 1e-4
        assert dirs[i] == dd
    assert min(xs) < 0.5 and max(xs) > 14.5  # sweeps the box
